"""Where the reference tree is present, compare its HostNMF with the oracle on fresh shapes."""
import numpy as np
import pytest

import oracle
from gpumlib_gb300 import inputs

pytestmark = pytest.mark.skipif(oracle.ref() is None, reason="reference HostNMF not built on this machine")


@pytest.mark.parametrize("rule", [0, 1])
@pytest.mark.parametrize("shape", [(19, 7, 2), (64, 64, 8), (130, 33, 11)])
@pytest.mark.parametrize("updateW", [True, False])
def test_reference_equals_oracle(rule, shape, updateW):
    n, m, r = shape
    V = inputs.uniform_matrix(100 + n, n, m)
    W, H = inputs.factors(200 + m, n, m, r)
    a = oracle.reference_run(rule, V, W, H, 6, updateW=updateW)
    b = oracle.hostnmf_run(rule, V, W, H, 6, updateW=updateW, eps=1e-8, nthreads=3)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
