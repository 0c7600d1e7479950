"""gpunmf_residual_fp64_noalloc: the relative residual for callers that cannot allocate.

The entry point takes caller-owned device matrices and keeps its scratch in a
fixed array inside the library, so it never calls cudaMalloc.  It is checked
through the C ABI against the job-based gpunmf_residual_fp64 (the existing
entry point, which allocates its workspaces at job creation) on two calls in
a row: a larger shape first, then a smaller one, so the second call runs with
the first call's partial sums still in the shared scratch array.  Each result
is also checked against the CPU oracle's residual (all in FP64), so the check
does not rest on the two entry points sharing their reduction code.  The bound
is the 1e-5 used for residuals elsewhere in these tests.
"""
import ctypes

import numpy as np
import pytest

import oracle
from gpumlib_gb300 import _native, inputs

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _device_colmajor(torch, a):
    flat = np.ascontiguousarray(np.asarray(a, dtype=np.float32).ravel(order="F"))
    return torch.from_numpy(flat).cuda()


def test_noalloc_residual_matches_job_residual_twice(gpu):
    torch = pytest.importorskip("torch")
    lib = _native.load()
    for n, m, r, vseed, fseed in ((1500, 1200, 24, 81, 82), (333, 257, 7, 83, 84)):
        V = inputs.uniform_matrix(vseed, n, m)
        W, H = inputs.factors(fseed, n, m, r)
        with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H) as nmf:
            expected = nmf.Residual()
        dV, dW, dH = (_device_colmajor(torch, a) for a in (V, W, H))
        out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        st = lib.gpunmf_residual_fp64_noalloc(n, m, r, ctypes.c_void_p(dV.data_ptr()),
                                              ctypes.c_void_p(dW.data_ptr()), ctypes.c_void_p(dH.data_ptr()),
                                              ctypes.c_void_p(out.data_ptr()), None)
        _native.check(st)
        torch.cuda.synchronize()
        got = out.item()
        assert abs(got - expected) <= TOL, (n, m, r, got, expected)
        assert abs(got - oracle.residual(V, W, H)) <= TOL, (n, m, r, got)


def test_noalloc_rejects_shapes_beyond_its_scratch(gpu):
    torch = pytest.importorskip("torch")
    lib = _native.load()
    small = torch.zeros(4, dtype=torch.float32, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(small.data_ptr())
    # 40000 x 40000 needs 313 * 313 = 97969 partial sums; the fixed scratch holds 65536.
    # The size check comes before any launch, so the small buffers are never read.
    st = lib.gpunmf_residual_fp64_noalloc(40000, 40000, 8, p, p, p, ctypes.c_void_p(out.data_ptr()), None)
    assert st == 1
    assert b"fixed scratch" in lib.gpunmf_last_error()
