"""Bounded device waits and the grid limit of the tensor-core kernels.

1. A wait that runs out.  The fused BF16 kernels' CTAs wait on one another (a
   tile's partial products, grid-wide sums), each wait bounded.  The test
   shortens the bound to about a millisecond and starts one tile's arrival
   counter one below zero from the host, so the fused update's wait for that
   tile cannot complete: the kernel must set its error word and return, the
   host must report GPUNMF_ERR_TIMEOUT, the job must destroy cleanly, and a
   fresh job afterwards must match the exact emulation.  No GPU fault is made:
   the failure is a counter that never reaches its target, and the wait that
   watches it ends on its own.
2. The grid limit.  With the kernels capped at 7 CTAs, every CTA of the fused
   Euclidean and KL kernels updates several chunks of factor rows in its tail
   (more than 64 rows per CTA in the Euclidean kernel, more than 128 in the KL
   kernel), which the full grid only does at much larger shapes.  One iteration
   is checked against the exact emulation (2e-5 relative Frobenius).
"""
import numpy as np
import pytest

from conftest import rel
from gpumlib_gb300 import _native, inputs
from test_gpu_bf16 import emulate_one
from test_gpu_kl_bf16 import emulate_kl_one

pytestmark = pytest.mark.gpu

TIMEOUT = 6
UNSUPPORTED = 4
SHORT_WAIT = 2_000_000  # SM clock cycles: about 1 ms at 2 GHz


def _kl_data(n, m, seed):
    g = np.random.Generator(np.random.PCG64(seed))
    return np.asfortranarray(g.poisson(2.0, size=(n, m)).astype(np.float32))


@pytest.mark.parametrize("rule", [0, 1], ids=["euclidean", "kl"])
def test_wait_runs_out_reports_timeout_and_engine_recovers(gpu, rule):
    lib = _native.load()
    n, m, r = 1536, 1024, 64  # both half-steps take the fused kernels at this shape
    V = inputs.uniform_matrix(91, n, m) if rule == 0 else _kl_data(n, m, 91)
    W, H = inputs.factors(92, n, m, r)
    nmf = gpu.make(rule, V, W, H, eps=1e-9, precision="bf16", quality_interval=0)
    try:
        nmf.Iterate(2)
        nmf.Synchronize()  # healthy so far
        _native.check(lib.gpunmf_set_wait_limit_cycles(nmf._h, SHORT_WAIT))
        _native.check(lib.gpunmf_inject_missing_arrival(nmf._h))
        nmf.Iterate(2)  # enqueues; the waits run out on the device
        st = lib.gpunmf_synchronize(nmf._h)
        assert st == TIMEOUT, (st, _native.last_error())
        assert "gave up waiting" in _native.last_error()
    finally:
        assert lib.gpunmf_destroy(nmf._h) == 0
        nmf._h = None
    # the engine (and the GPU context) is usable: a fresh job gives the exact emulation's result
    eps = np.float32(1e-9)
    with gpu.make(rule, V, W, H, eps=eps, precision="bf16", quality_interval=0) as fresh:
        fresh.DoIteration()
        W1g, H1g = fresh.GetW(), fresh.GetH()
    emulate = emulate_one if rule == 0 else emulate_kl_one
    W1, H1 = emulate(V, W, H, float(eps), H1g)
    assert rel(H1g, H1) <= 2e-5 and rel(W1g, W1) <= 2e-5


def test_injection_needs_a_fused_job(gpu):
    lib = _native.load()
    n, m, r = 300, 200, 8
    V = inputs.uniform_matrix(93, n, m)
    W, H = inputs.factors(94, n, m, r)
    with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H, precision="fp32") as nmf:
        assert lib.gpunmf_inject_missing_arrival(nmf._h) == UNSUPPORTED
        assert lib.gpunmf_set_wait_limit_cycles(nmf._h, SHORT_WAIT) == UNSUPPORTED


@pytest.mark.parametrize("rule", [0, 1], ids=["euclidean", "kl"])
def test_capped_grid_multi_chunk_tails_match_emulation(gpu, rule):
    lib = _native.load()
    n, m, r = 4096, 2048, 64
    V = inputs.uniform_matrix(95, n, m) if rule == 0 else _kl_data(n, m, 95)
    W, H = inputs.factors(96, n, m, r)
    eps = np.float32(1e-9)
    _native.check(lib.gpunmf_set_grid_limit(7))
    try:
        # 7 CTAs: 292 rows of H and 585 rows of W per CTA
        with gpu.make(rule, V, W, H, eps=eps, precision="bf16", quality_interval=0) as nmf:
            nmf.DoIteration()
            W1g, H1g = nmf.GetW(), nmf.GetH()
    finally:
        _native.check(lib.gpunmf_set_grid_limit(0))
    emulate = emulate_one if rule == 0 else emulate_kl_one
    W1, H1 = emulate(V, W, H, float(eps), H1g)
    assert rel(H1g, H1) <= 2e-5, "H-step with multi-chunk tails differs"
    assert rel(W1g, W1) <= 2e-5, "W-step with multi-chunk tails differs"
