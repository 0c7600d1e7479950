"""Additive update rules on the GPU (nmf_additive_euclidian.cpp:29-57,
nmf_additive_divergence.cpp:29-51, nmf_kernels.cu:31-38,
nmf_kernels_additive_divergence.cu:39-185).

The golden cases of both additive rules (the reference's HostNMF, both
factors updated) run in test_gpu_fp32_parity.py.  Here:
1. the fixed-H form of NMF_AdditiveEuclidian (what the reference's GPU class
   runs: its H step writes into a workspace) keeps H bit-identical and
   tracks the oracle's W within the FP32 bound;
2. odd shapes and updateW=False against the float oracle;
3. the BF16 tensor-core path of the additive rules tracks the FP32 path
   (final relative residuals within 1e-3);
4. the kernel-level entry points against an FP64 statement of their formulas.
"""
import ctypes

import numpy as np
import pytest

import oracle
from conftest import rel
from gpumlib_gb300 import _native, inputs

pytestmark = pytest.mark.gpu

TOL = 1e-4


def run(g, rule, V, W, H, iters, updateW=True, precision="fp32", eps=1e-8):
    with g.make(rule, V, W, H, eps=eps, precision=precision) as nmf:
        nmf.Iterate(iters, updateW)
        return nmf.GetW(), nmf.GetH(), nmf.Residual()


@pytest.mark.parametrize("shape", [(200, 150, 6), (37, 23, 3), (1000, 777, 20), (1, 40, 1)])
def test_fixed_h_is_the_reference_gpu_class(gpu, shape):
    n, m, r = shape
    V = inputs.uniform_matrix(80 + n, n, m)
    W, H = inputs.factors(81 + m, n, m, r)
    with gpu.NMF_AdditiveEuclidian(V, W, H) as nmf:   # default: the reference GPU class's behaviour
        nmf.Iterate(10)
        Wg, Hg = nmf.GetW(), nmf.GetH()
    assert np.array_equal(Hg, H), "the fixed-H rule must leave H untouched"
    Wo, Ho = oracle.hostnmf_run(2, V, W, H, 10, skip_h=True, nthreads=8)
    assert np.array_equal(Ho, H)
    assert rel(Wg, Wo) <= TOL


@pytest.mark.parametrize("rule", [2, 3])
@pytest.mark.parametrize("shape", [(129, 257, 65), (1, 1, 1), (300, 1, 3), (1500, 700, 40)])
def test_additive_odd_shapes_vs_oracle(gpu, rule, shape):
    n, m, r = shape
    V = inputs.uniform_matrix(90 + n, n, m)
    W, H = inputs.factors(91 + m, n, m, r)
    Wg, Hg, _ = run(gpu, rule, V, W, H, 6)
    Wo, Ho = oracle.hostnmf_run(rule, V, W, H, 6, clamp_sums=True, nthreads=8)
    assert rel(Wg.astype(np.float64) @ Hg, Wo.astype(np.float64) @ Ho) <= TOL
    assert np.all(Wg >= 0) and np.all(Hg >= 0)


@pytest.mark.parametrize("rule", [2, 3])
def test_additive_update_w_false(gpu, rule):
    n, m, r = 230, 170, 7
    V = inputs.uniform_matrix(95, n, m)
    W, H = inputs.factors(96, n, m, r)
    Wg, Hg, _ = run(gpu, rule, V, W, H, 4, updateW=False)
    assert np.array_equal(Wg, W)
    _, Ho = oracle.hostnmf_run(rule, V, W, H, 4, updateW=False, clamp_sums=True, nthreads=8)
    assert rel(Hg, Ho) <= TOL


@pytest.mark.parametrize("rule,shape", [(2, (2048, 1536, 32)), (4, (2048, 1536, 32)), (3, (1024, 2048, 64)),
                                        (2, (1000, 777, 100)), (3, (513, 700, 7))])
def test_additive_bf16_tracks_fp32(gpu, rule, shape):
    n, m, r = shape
    V = inputs.lowrank_gamma(n, m, r, 2.0, 0.5, seed=97)
    W, H = inputs.factors(98, n, m, r)
    iters = 60
    _, _, r32 = run(gpu, rule, V, W, H, iters, eps=1e-9)
    Wb, Hb, r16 = run(gpu, rule, V, W, H, iters, precision="bf16", eps=1e-9)
    assert abs(r16 - r32) <= 1e-3, (r16, r32)
    assert np.all(Wb >= 0) and np.all(Hb >= 0)
    if rule == 4:
        assert np.array_equal(Hb, H)


def test_additive_deterministic(gpu):
    n, m, r = 600, 500, 24
    V = inputs.uniform_matrix(99, n, m)
    W, H = inputs.factors(100, n, m, r)
    for rule in (2, 3, 4):
        for prec in ("fp32", "bf16"):
            a = run(gpu, rule, V, W, H, 5, precision=prec)
            b = run(gpu, rule, V, W, H, 5, precision=prec)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


# ---------------------------------------------------------------------------
# kernel-level entry points (torch holds the device memory)
# ---------------------------------------------------------------------------
torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float32).ravel(order="F"))).cuda()


def ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_additive_euclidean_entry_point(gpu):
    lib = _native.load()
    g = np.random.Generator(np.random.PCG64(2))
    count = 10009
    x, d1, d2 = (g.random(count, dtype=np.float32) + np.float32(0.05) for _ in range(3))
    tx, t1, t2 = dev(x), dev(d1), dev(d2)
    assert lib.gpumlib_cuda_nmf_additive_euclidean_update_matrix(20, 512, ptr(tx), ptr(t1), ptr(t2), count) == 0
    torch.cuda.synchronize()
    xd = x.astype(np.float64)
    exp = np.maximum(xd + (xd / d2) * (d1.astype(np.float64) - d2), 0.0)
    got = tx.cpu().numpy()
    assert np.all(got >= 0)
    np.testing.assert_allclose(got, exp, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("which", ["h", "w"])
def test_additive_kl_entry_points(gpu, which):
    lib = _native.load()
    n, m, r = 301, 203, 13
    V = inputs.uniform_matrix(10, n, m)
    W, H = inputs.factors(11, n, m, r)
    WH = oracle.hostnmf_wh(W, H)
    tv, tw, th, twh = dev(V), dev(W), dev(H), dev(WH)
    Vd, Wd, Hd = (a.astype(np.float64) for a in (V, W, H))
    Rm1 = Vd / (WH.astype(np.float64) + 1e-8) - 1.0
    d3 = _native.Dim3(1, 1, 1)
    if which == "h":
        sums = np.maximum(Wd.sum(axis=0), 1e-8).astype(np.float32)
        ts = dev(sums)
        assert lib.gpumlib_cuda_nmf_additive_divergence_update_matrix_h(
            d3, d3, ptr(th), ptr(tw), ptr(tv), ptr(twh), ptr(ts), n, m, r) == 0
        torch.cuda.synchronize()
        got = th.cpu().numpy().reshape(m, r).T
        exp = np.maximum(Hd + Hd / sums[:, None] * (Wd.T @ Rm1), 0.0)
    else:
        sums = np.maximum(Hd.sum(axis=1), 1e-8).astype(np.float32)
        ts = dev(sums)
        assert lib.gpumlib_cuda_nmf_additive_divergence_update_matrix_w(
            d3, d3, ptr(tw), ptr(th), ptr(tv), ptr(twh), ptr(ts), n, m, r) == 0
        torch.cuda.synchronize()
        got = tw.cpu().numpy().reshape(r, n).T
        exp = np.maximum(Wd + Wd / sums[None, :] * (Rm1 @ Hd.T), 0.0)
    assert rel(got, exp) <= 2e-5
