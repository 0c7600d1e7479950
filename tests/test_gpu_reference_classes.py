"""The engine against the reference's own GPU implementation, run on the same GPU.

oracle/build.py compiles the reference's GPU NMF classes and kernels from its sources
(nmf_multiplicative_euclidian.cpp:29-67, nmf_multiplicative_divergence.cpp:29-50,
nmf_kernels.cu, nmf_kernels_quality.cu, DeviceMatrix.h's cublasSgemm products) for sm_103a
into oracle/_ref/libref_gpu_nmf.so, from the reference tree or its staged copy; these
tests skip where neither is present.

- Classes: the reference's NMF_MultiplicativeEuclidianDistance / NMF_MultiplicativeDivergence
  constructed from (V, W, H) and the engine's FP32 path (the drop-in), same seeded inputs and
  iterations, epsilon 1e-8 (the reference's SMALL_VALUE_TO_ADD_DENOMINATOR): W, H and W H
  within 1e-4 relative Frobenius, at small and odd shapes and at the benchmark shapes.
- Shapes whose reference reductions would run with 32 threads or fewer (KL with n or m <= 32)
  are not run: those reference kernels read past their shared memory there (the shim refuses
  them).
- Kernel-level API: the reference's own kernels and the engine's entry points of the same
  names on the same device buffers: the multiplicative Euclidean update bit for bit, the KL
  updates, the column / row sums and the quality within float rounding of their different
  summation orders.
"""
import ctypes

import numpy as np
import pytest

import oracle
from conftest import rel
from gpumlib_gb300 import _native, inputs

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1e-4


@pytest.fixture(scope="module")
def refgpu(gpu):
    lib = oracle.reference_gpu()
    if lib is None:
        pytest.skip("the reference's GPU sources are not present (reference tree or staged copy)")
    assert lib.refgpu_init() == 0
    return lib


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float32).ravel(order="F"))).cuda()


def ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def kl_counts(seed, n, m):
    g = np.random.Generator(np.random.PCG64(seed))
    return np.asfortranarray(g.poisson(2.0, size=(n, m)).astype(np.float32))


CASES = [
    # name, rule, n, m, r, iters
    ("euclid_1024x768_r16", 0, 1024, 768, 16, 20),
    ("euclid_odd_37x23_r3", 0, 37, 23, 3, 25),
    ("euclid_tall_3001x257_r33", 0, 3001, 257, 33, 10),
    ("kl_1024x768_r16", 1, 1024, 768, 16, 20),
    ("kl_odd_65x47_r5", 1, 65, 47, 5, 15),
    ("kl_wide_257x3001_r40", 1, 257, 3001, 40, 10),
    ("euclid_8192x8192_r64", 0, 8192, 8192, 64, 3),
    ("kl_16384x4096_r128", 1, 16384, 4096, 128, 2),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_engine_fp32_matches_reference_gpu_classes(gpu, refgpu, case):
    name, rule, n, m, r, iters = case
    V = inputs.uniform_matrix(200 + n % 97, n, m) if rule == 0 else kl_counts(300 + m % 89, n, m)
    W, H = inputs.factors(400 + r, n, m, r)
    Wr, Hr, _ = oracle.reference_gpu_run(rule, V, W, H, iters)
    with gpu.make(rule, V, W, H, eps=1e-8, precision="fp32", quality_interval=0) as nmf:
        nmf.Iterate(iters)
        Wg, Hg = nmf.GetW(), nmf.GetH()
    assert rel(Wg, Wr) <= TOL and rel(Hg, Hr) <= TOL
    if n * m <= 4_000_000:
        assert rel(Wg.astype(np.float64) @ Hg, Wr.astype(np.float64) @ Hr) <= TOL
    else:   # W H on a sample of columns
        cols = np.arange(0, m, 61)
        assert rel(Wg.astype(np.float64) @ Hg[:, cols], Wr.astype(np.float64) @ Hr[:, cols]) <= TOL


def test_euclidean_update_kernel_bit_for_bit(gpu, refgpu):
    lib = _native.load()
    g = np.random.Generator(np.random.PCG64(11))
    count = 100_003
    nm, dm, x = (g.random(count, dtype=np.float32) for _ in range(3))
    dm[::7] = 0.0   # the epsilon guard
    tn, td = dev(nm), dev(dm)
    ours, theirs = dev(x), dev(x)
    blocks = (count + 511) // 512
    assert lib.gpumlib_cuda_nmf_multiplicative_euclidean_update_matrix(blocks, 512, ptr(tn), ptr(td), ptr(ours),
                                                                       count) == 0
    assert refgpu.gpumlib_cuda_nmf_multiplicative_euclidean_update_matrix(blocks, 512, ptr(tn), ptr(td),
                                                                          ptr(theirs), count) == 0
    torch.cuda.synchronize()
    assert torch.equal(ours.view(torch.int32), theirs.view(torch.int32))


def test_sum_and_quality_kernels_match_reference_kernels(gpu, refgpu):
    lib = _native.load()
    n, m, r = 1517, 933, 19
    V = inputs.uniform_matrix(12, n, m)
    W, H = inputs.factors(13, n, m, r)
    W[:, 3] = 0.0   # the sums' epsilon clamp
    tw, th = dev(W), dev(H)
    for ours_fn, ref_fn, t, a, b in ((lib.gpumlib_nmf_sum_w, refgpu.refgpu_kernel_sum_w, tw, n, r),
                                     (lib.gpumlib_nmf_sum_h, refgpu.refgpu_kernel_sum_h, th, r, m)):
        so, sr = torch.zeros(r, device="cuda"), torch.zeros(r, device="cuda")
        assert ours_fn(1024, ptr(t), a, b, ptr(so)) == 0
        assert ref_fn(1024, ptr(t), a, b, ptr(sr)) == 0
        torch.cuda.synchronize()
        np.testing.assert_allclose(so.cpu().numpy(), sr.cpu().numpy(), rtol=2e-6)
    WH = oracle.hostnmf_wh(W, H)
    tv, twh = dev(V), dev(WH)
    qo, qr = torch.zeros(1, device="cuda"), torch.zeros(1, device="cuda")
    assert lib.gpumlib_nmf_quality(1024, ptr(tv), ptr(twh), n * m, ptr(qo)) == 0
    assert refgpu.refgpu_kernel_quality(1024, ptr(tv), ptr(twh), n * m, ptr(qr)) == 0
    torch.cuda.synchronize()
    # the reference sums 1.4M terms in float per thread and in a float tree; the engine in FP64
    assert abs(qo.item() - qr.item()) <= 1e-4 * abs(qr.item())


@pytest.mark.parametrize("which", ["h", "w"])
def test_kl_update_kernels_match_reference_kernels(gpu, refgpu, which):
    lib = _native.load()
    n, m, r = 701, 517, 21
    V = kl_counts(14, n, m)
    W, H = inputs.factors(15, n, m, r)
    WH = oracle.hostnmf_wh(W, H)
    tv, twh = dev(V), dev(WH)
    Wd, Hd = W.astype(np.float64), H.astype(np.float64)
    d3 = _native.Dim3(1, 1, 1)
    if which == "h":
        sums = dev(np.maximum(Wd.sum(axis=0), 1e-8))
        ours, theirs, other = dev(H), dev(H), dev(W)
        grid, block = _native.Dim3((m + 31) // 32, (r + 31) // 32, 1), _native.Dim3(32, 16, 1)   # nmf_multiplicative_divergence.h:51
        assert lib.gpumlib_cuda_nmf_multiplicative_divergence_update_matrix_h(
            d3, d3, ptr(ours), ptr(other), ptr(tv), ptr(twh), ptr(sums), n, m, r) == 0
        assert refgpu.gpumlib_cuda_nmf_multiplicative_divergence_update_matrix_h(
            grid, block, ptr(theirs), ptr(other), ptr(tv), ptr(twh), ptr(sums), n, m, r) == 0
    else:
        sums = dev(np.maximum(Hd.sum(axis=1), 1e-8))
        ours, theirs, other = dev(W), dev(W), dev(H)
        grid, block = _native.Dim3((r + 31) // 32, (n + 31) // 32, 1), _native.Dim3(16, 32, 1)
        assert lib.gpumlib_cuda_nmf_multiplicative_divergence_update_matrix_w(
            d3, d3, ptr(ours), ptr(other), ptr(tv), ptr(twh), ptr(sums), n, m, r) == 0
        assert refgpu.gpumlib_cuda_nmf_multiplicative_divergence_update_matrix_w(
            grid, block, ptr(theirs), ptr(other), ptr(tv), ptr(twh), ptr(sums), n, m, r) == 0
    torch.cuda.synchronize()
    np.testing.assert_allclose(ours.cpu().numpy(), theirs.cpu().numpy(), rtol=2e-5)
