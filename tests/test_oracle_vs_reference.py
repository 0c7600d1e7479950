"""Where the reference tree is present, compare its HostNMF with the oracle on fresh shapes."""
import numpy as np
import pytest

import oracle
from gpumlib_gb300 import inputs

pytestmark = pytest.mark.skipif(oracle.ref() is None, reason="reference HostNMF not built on this machine")


@pytest.mark.parametrize("rule", [0, 1, 2, 3])
@pytest.mark.parametrize("shape", [(19, 7, 2), (64, 64, 8), (130, 33, 11)])
@pytest.mark.parametrize("updateW", [True, False])
def test_reference_equals_oracle(rule, shape, updateW):
    n, m, r = shape
    V = inputs.uniform_matrix(100 + n, n, m)
    W, H = inputs.factors(200 + m, n, m, r)
    a = oracle.reference_run(rule, V, W, H, 6, updateW=updateW)
    b = oracle.hostnmf_run(rule, V, W, H, 6, updateW=updateW, eps=1e-8, nthreads=3)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def same_bits(a, b):
    """Bit for bit, NaN matching NaN (the payload of 0/0 is not part of the arithmetic)."""
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    return a.shape == b.shape and bool(np.all((a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))))


EDGE_SHAPES = [(1, 5, 1), (5, 1, 1), (17, 13, 1), (6, 4, 9), (2, 2, 2)]


@pytest.mark.parametrize("rule", [0, 1, 2, 3])
@pytest.mark.parametrize("shape", EDGE_SHAPES, ids=["%dx%dr%d" % s for s in EDGE_SHAPES])
def test_reference_equals_oracle_edge_shapes(rule, shape):
    """One row or column, rank 1, rank above both sides; the multiplicative (0, 1) and additive (2, 3)
    rules of HostNMF.h:64-233."""
    n, m, r = shape
    V = inputs.uniform_matrix(300 + n, n, m)
    W, H = inputs.factors(400 + m, n, m, r)
    a = oracle.reference_run(rule, V, W, H, 5)
    b = oracle.hostnmf_run(rule, V, W, H, 5, eps=1e-8, nthreads=2)
    assert same_bits(a[0], b[0]) and same_bits(a[1], b[1])


@pytest.mark.parametrize("rule", [0, 1, 2, 3])
def test_reference_equals_oracle_with_zeros(rule):
    """V with a zero row, a zero column and scattered exact zeros; W with a zero column (the CPU KL
    rule has no eps on its sums, so that column's H row becomes 0/0 there: NaN in both)."""
    n, m, r = 40, 30, 5
    V = inputs.uniform_matrix(17, n, m)
    V[3, :] = 0.0
    V[:, 7] = 0.0
    V[::5, ::3] = 0.0
    W, H = inputs.factors(18, n, m, r)
    W[:, 2] = 0.0
    a = oracle.reference_run(rule, V, W, H, 4)
    b = oracle.hostnmf_run(rule, V, W, H, 4, eps=1e-8, nthreads=3)
    assert same_bits(a[0], b[0]) and same_bits(a[1], b[1])
    if rule == 1:
        assert np.isnan(b[1][2]).all()
