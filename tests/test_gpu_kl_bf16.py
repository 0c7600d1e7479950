"""BF16 tensor-core path of the KL rule (fused S = WH -> R = V/(S+eps) -> numerator).

1. One iteration against an exact emulation: S from BF16-rounded W and H, R = V_bf16/(S+eps) rounded to
   BF16, numerators from R and the BF16 factor, denominators max(sum, eps) in FP32 -> the GPU result may
   differ only by accumulation order (bound 2e-5 relative Frobenius).
2. Over many iterations it tracks the FP32 KL path (residuals within 1e-3) and the FP64 oracle.
"""
import numpy as np
import pytest

import oracle
from conftest import rel
from gpumlib_gb300 import inputs
from test_gpu_bf16 import bf16

pytestmark = pytest.mark.gpu


def emulate_kl_one(V, W, H, eps, H1_gpu):
    Vb, Wb, Hb = bf16(V), bf16(W), bf16(H)
    Wd, Hd = W.astype(np.float64), H.astype(np.float64)
    S = Wb @ Hb
    R = bf16((Vb / (S + eps)).astype(np.float32))
    sw = np.maximum(Wd.sum(axis=0), eps)
    H1 = Hd * (Wb.T @ R) / sw[:, None]
    H1b = bf16(H1_gpu)
    S2 = Wb @ H1b
    R2 = bf16((Vb / (S2 + eps)).astype(np.float32))
    sh = np.maximum(H1_gpu.astype(np.float64).sum(axis=1), eps)
    W1 = Wd * (R2 @ H1b.T) / sh[None, :]
    return W1, H1


SHAPES = [(512, 384, 16), (1000, 777, 20), (300, 1300, 7), (129, 65, 1), (2048, 1024, 128), (513, 700, 100),
          (64, 4096, 64), (37, 11, 3),
          # ranks whose padded width (48, 80, 96) fills the factor tile's second 64-column box only in part
          (700, 900, 40), (1030, 640, 70), (400, 1500, 90)]


@pytest.mark.parametrize("shape", SHAPES, ids=["%dx%dr%d" % s for s in SHAPES])
def test_kl_one_iteration_matches_emulation(gpu, shape):
    n, m, r = shape
    g = np.random.Generator(np.random.PCG64(n + m + r))
    V = np.asfortranarray(g.poisson(2.0, size=(n, m)).astype(np.float32))
    W, H = inputs.factors(90 + n, n, m, r)
    eps = np.float32(1e-9)
    with gpu.NMF_MultiplicativeDivergence(V, W, H, eps=eps, precision="bf16", quality_interval=0) as nmf:
        nmf.DoIteration()
        W1g, H1g = nmf.GetW(), nmf.GetH()
    W1, H1 = emulate_kl_one(V, W, H, float(eps), H1g)
    assert rel(H1g, H1) <= 2e-5, "H-step (fused KL tcgen05) differs"
    assert rel(W1g, W1) <= 2e-5, "W-step (fused KL tcgen05) differs"


@pytest.mark.parametrize("shape", [(129, 65, 1), (300, 1300, 7), (1000, 777, 20)], ids=["129x65r1", "300x1300r7", "1000x777r20"])
def test_kl_tiny_eps_matches_emulation(gpu, shape):
    """eps = 1e-30: in the zero-padded rows and columns of a tile (S = 0) a pair's product of
    S + eps underflows, so the kernel's one-reciprocal-per-pair step must fall back to plain
    divisions there; any inf or NaN it let through would reach the numerators."""
    n, m, r = shape
    g = np.random.Generator(np.random.PCG64(3 * n + m + r))
    V = np.asfortranarray(g.poisson(2.0, size=(n, m)).astype(np.float32))
    W, H = inputs.factors(190 + n, n, m, r)
    eps = np.float32(1e-30)
    with gpu.NMF_MultiplicativeDivergence(V, W, H, eps=eps, precision="bf16", quality_interval=0) as nmf:
        nmf.DoIteration()
        W1g, H1g = nmf.GetW(), nmf.GetH()
    assert np.isfinite(W1g).all() and np.isfinite(H1g).all()
    W1, H1 = emulate_kl_one(V, W, H, float(eps), H1g)
    assert rel(H1g, H1) <= 2e-5, "H-step (fused KL tcgen05) differs"
    assert rel(W1g, W1) <= 2e-5, "W-step (fused KL tcgen05) differs"


@pytest.mark.parametrize("shape", [(1500, 900, 128), (1024, 700, 40)], ids=["1500x900r128", "1024x700r40"])
def test_kl_sparse_counts_match_emulation(gpu, shape):
    """Count data with ~90% zeros (the sparse count workload: lambda = 0.01 P Q with P, Q ~ Gamma(0.3, 1)):
    most ratios V / (S + eps) are exactly 0, the rest large; one iteration against the emulation."""
    n, m, r = shape
    g = np.random.Generator(np.random.PCG64(5 * n + m))
    P = g.gamma(0.3, 1.0, size=(n, 64))
    Q = g.gamma(0.3, 1.0, size=(64, m))
    V = np.asfortranarray(g.poisson(0.01 * (P @ Q)).astype(np.float32))
    assert np.mean(V == 0) > 0.8
    W, H = inputs.factors(290 + n, n, m, r)
    eps = np.float32(1e-9)
    with gpu.NMF_MultiplicativeDivergence(V, W, H, eps=eps, precision="bf16", quality_interval=0) as nmf:
        nmf.DoIteration()
        W1g, H1g = nmf.GetW(), nmf.GetH()
    W1, H1 = emulate_kl_one(V, W, H, float(eps), H1g)
    assert rel(H1g, H1) <= 2e-5, "H-step (fused KL tcgen05) differs"
    assert rel(W1g, W1) <= 2e-5, "W-step (fused KL tcgen05) differs"


def test_kl_bf16_tracks_fp32(gpu):
    n, m, r = 2048, 1536, 64
    g = np.random.Generator(np.random.PCG64(7))
    P = g.gamma(0.3, 1.0, size=(n, 64))
    Q = g.gamma(0.3, 1.0, size=(64, m))
    V = np.asfortranarray(g.poisson(P @ Q).astype(np.float32))
    W, H = inputs.factors(8, n, m, r)
    res = {}
    for prec in ("fp32", "bf16"):
        with gpu.NMF_MultiplicativeDivergence(V, W, H, eps=1e-9, precision=prec, quality_interval=0) as nmf:
            nmf.Iterate(100)
            res[prec] = (nmf.Residual(), nmf.ObjectiveKL())
    assert abs(res["bf16"][0] - res["fp32"][0]) <= 1e-3, res
    assert abs(res["bf16"][1] - res["fp32"][1]) <= 1e-3 * abs(res["fp32"][1]), res


def test_kl_bf16_error_vs_f64_oracle(gpu):
    n, m, r = 700, 500, 12
    g = np.random.Generator(np.random.PCG64(9))
    V = np.asfortranarray(g.poisson(3.0, size=(n, m)).astype(np.float32))
    W, H = inputs.factors(10, n, m, r)
    with gpu.NMF_MultiplicativeDivergence(V, W, H, eps=1e-9, precision="bf16", quality_interval=0) as nmf:
        nmf.Iterate(20)
        Wg, Hg = nmf.GetW(), nmf.GetH()
    Wd, Hd = oracle.f64_run(1, V, W, H, 20, eps=1e-9, nthreads=8)
    assert rel(Wg.astype(np.float64) @ Hg, Wd @ Hd) <= 5e-3


def test_kl_bf16_update_w_false_and_deterministic(gpu):
    n, m, r = 900, 600, 32
    g = np.random.Generator(np.random.PCG64(11))
    V = np.asfortranarray(g.poisson(1.5, size=(n, m)).astype(np.float32))
    W, H = inputs.factors(12, n, m, r)
    outs = []
    for _ in range(2):
        with gpu.NMF_MultiplicativeDivergence(V, W, H, precision="bf16", quality_interval=0) as nmf:
            nmf.Iterate(3)
            nmf.DoIteration(updateW=False)
            outs.append((nmf.GetW(), nmf.GetH()))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_kl_headline_shape_one_iteration_matches_emulation(gpu):
    """The KL benchmark workload itself (V 16384 x 4096 Poisson counts, r = 128, eps 1e-9): one BF16
    iteration of the fused KL kernels against the exact emulation on 768 columns of H and 768 rows of
    W (the emulated products of the whole matrices would take minutes on the host); bound 2e-5."""
    from test_gpu_bf16 import _slice_index
    cfg = inputs.kl_counts()
    V, W, H, eps = cfg["V"], cfg["W"], cfg["H"], np.float32(cfg["eps"])
    with gpu.NMF_MultiplicativeDivergence(V, W, H, eps=eps, precision="bf16", quality_interval=0) as nmf:
        nmf.DoIteration()
        W1g, H1g = nmf.GetW(), nmf.GetH()
    e = float(eps)
    n, m = V.shape
    cols = _slice_index(m, 3)
    rows = _slice_index(n, 4)
    Wb, Hb = bf16(W), bf16(H)
    Wd, Hd = W.astype(np.float64), H.astype(np.float64)
    S = Wb @ Hb[:, cols]
    R = bf16((bf16(V[:, cols]) / (S + e)).astype(np.float32))
    sw = np.maximum(Wd.sum(axis=0), e)
    H1 = Hd[:, cols] * (Wb.T @ R) / sw[:, None]
    assert rel(H1g[:, cols], H1) <= 2e-5, "H-step (fused KL kernel) differs at 16384x4096 r=128"
    H1b = bf16(H1g)
    S2 = Wb[rows] @ H1b
    R2 = bf16((bf16(V[rows, :]) / (S2 + e)).astype(np.float32))
    sh = np.maximum(H1g.astype(np.float64).sum(axis=1), e)
    W1 = Wd[rows] * (R2 @ H1b.T) / sh[None, :]
    assert rel(W1g[rows], W1) <= 2e-5, "W-step (fused KL kernel) differs at 16384x4096 r=128"
