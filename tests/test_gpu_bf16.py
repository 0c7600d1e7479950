"""BF16 tensor-core path (tcgen05 + TMA) of the Euclidean rule.

1. One iteration against an exact emulation: the numerators W'V and VH' are
   formed in FP64 from BF16-rounded operands (what the tensor cores see),
   the denominators in FP64 from the FP32 factors; the GPU result may differ
   only by FP32 accumulation order (bound 2e-5 relative Frobenius).
2. Over many iterations the BF16 path tracks the FP32 path: final relative
   residuals within 1e-3 (the acceptance bound between the two paths).
"""
import numpy as np
import pytest

import oracle
from conftest import rel
from gpumlib_gb300 import inputs

pytestmark = pytest.mark.gpu


def bf16(a):
    """Round float32 to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def emulate_one(V, W, H, eps, H1_gpu):
    Vb, Wb = bf16(V), bf16(W)
    Wd, Hd = W.astype(np.float64), H.astype(np.float64)
    H1 = Hd * (Wb.T @ Vb) / ((Wd.T @ Wd) @ Hd + eps)
    Hg = H1_gpu.astype(np.float64)
    W1 = Wd * (Vb @ bf16(H1_gpu).T) / (Wd @ (Hg @ Hg.T) + eps)
    return W1, H1


# The last two run the fused half-step kernel with more than 64 factor rows per CTA in one half-step
# (20000 rows over 152 CTAs: three chunks in the update tail); the first one is not fused (19 stream-K
# segments per tile in its H-step, above the fused tail's 15).
SHAPES = [(8192, 1024, 64), (1000, 777, 20), (300, 1300, 7), (129, 65, 16), (64, 64, 1), (2048, 4096, 128),
          (513, 2047, 176), (37, 11, 3), (20000, 2048, 32), (2048, 20000, 64)]


@pytest.mark.parametrize("shape", SHAPES, ids=["%dx%dr%d" % s for s in SHAPES])
def test_one_iteration_matches_emulation(gpu, shape):
    n, m, r = shape
    V = inputs.uniform_matrix(50 + n, n, m)
    W, H = inputs.factors(60 + m, n, m, r)
    eps = np.float32(1e-9)
    with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H, eps=eps, precision="bf16", quality_interval=0) as nmf:
        nmf.DoIteration()
        W1g, H1g = nmf.GetW(), nmf.GetH()
    W1, H1 = emulate_one(V, W, H, float(eps), H1g)
    assert rel(H1g, H1) <= 2e-5, "H-step (tcgen05 W'V + update) differs"
    assert rel(W1g, W1) <= 2e-5, "W-step (tcgen05 VH' + update) differs"


def test_update_w_false_bf16(gpu):
    n, m, r = 700, 900, 32
    V = inputs.uniform_matrix(70, n, m)
    W, H = inputs.factors(71, n, m, r)
    with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H, precision="bf16", quality_interval=0) as nmf:
        nmf.DoIteration(updateW=False)
        nmf.DoIteration(updateW=False)
        assert np.array_equal(nmf.GetW(), W)
        H2 = nmf.GetH()
    Hd = H.astype(np.float64)
    Wd = W.astype(np.float64)
    G = Wd.T @ Wd
    num = bf16(W).T @ bf16(V)
    for _ in range(2):
        Hd = Hd * num / (G @ Hd + 1e-8)
    assert rel(H2, Hd) <= 2e-5


def test_bf16_deterministic(gpu):
    n, m, r = 1500, 1100, 48
    V = inputs.uniform_matrix(72, n, m)
    W, H = inputs.factors(73, n, m, r)
    outs = []
    for _ in range(2):
        with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H, precision="bf16", quality_interval=0) as nmf:
            nmf.Iterate(5)
            outs.append((nmf.GetW(), nmf.GetH()))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_bf16_tracks_fp32_residual(gpu):
    """Low-rank + noise data as in the 8192^2 workload, at 2048 x 2048: residuals agree within 1e-3."""
    n = m = 2048
    r = 64
    V = inputs.lowrank_gamma(n, m, 64, 2.0, 0.5, seed=2)
    W, H = inputs.factors(3, n, m, r)
    res = {}
    for prec in ("fp32", "bf16"):
        with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H, eps=1e-9, precision=prec, quality_interval=0) as nmf:
            nmf.Iterate(200)
            res[prec] = nmf.Residual()
    assert abs(res["bf16"] - res["fp32"]) <= 1e-3, res


def test_bf16_error_vs_f64_oracle(gpu):
    """Relative Frobenius error of W H against the FP64 CPU oracle after 30 iterations."""
    n, m, r = 1024, 768, 16
    V = inputs.lowrank_gamma(n, m, 16, 2.0, 0.5, seed=5)
    W, H = inputs.factors(6, n, m, r)
    with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H, eps=1e-9, precision="bf16", quality_interval=0) as nmf:
        nmf.Iterate(30)
        Wg, Hg = nmf.GetW(), nmf.GetH()
    Wd, Hd = oracle.f64_run(0, V, W, H, 30, eps=1e-9, nthreads=8)
    assert rel(Wg.astype(np.float64) @ Hg, Wd @ Hd) <= 5e-3


def test_bf16_quality_path(gpu):
    """The quality bookkeeping also runs on the BF16 path (FP32 fused W H reduction)."""
    n, m, r = 400, 300, 8
    V = inputs.uniform_matrix(74, n, m)
    W, H = inputs.factors(75, n, m, r)
    with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H, precision="bf16") as nmf:
        for _ in range(5):
            nmf.DoIteration()
        q = nmf.QualityImprovement()
    assert np.isfinite(q) and q != 1.0


@pytest.mark.parametrize("rule,shape", [(0, (2048, 1536, 64)), (0, (1000, 777, 20)), (1, (1024, 2048, 64)),
                                        (0, (300, 4100, 128))])
def test_bf16_quality_tracks_fp32(gpu, rule, shape):
    """BF16 jobs sample the quality on the tensor cores (W H from the BF16 factors, V as BF16): the
    lagged improvements (nmf_base.h:70-89) follow the FP32 job's over the first iterations."""
    n, m, r = shape
    V = inputs.lowrank_gamma(n, m, min(r, 16), 2.0, 0.5, seed=23)
    W, H = inputs.factors(24, n, m, r)
    seqs = {}
    for prec in ("fp32", "bf16"):
        with gpu.make(rule, V, W, H, eps=1e-9, precision=prec) as nmf:
            d = []
            for _ in range(8):
                nmf.DoIteration()
                d.append(nmf.QualityImprovement())
            seqs[prec] = np.array(d, dtype=np.float64)
    a, b = seqs["fp32"], seqs["bf16"]
    assert a[0] == b[0] == 1.0 and a[1] == b[1] == 1.0      # no improvement before the third sample
    scale = np.abs(a[2:]).max()
    assert np.abs(a[2:] - b[2:]).max() <= 2e-2 * scale, (a, b)


def test_two_jobs_interleaved_match_alone(gpu):
    """Two BF16 jobs with the fused half-step kernel, each on its own stream, iterated alternately:
    every launch follows one on the other stream, so the engine orders the two jobs' fused grids
    (their CTAs wait on one another, so two of them must not share the SMs).  The kernels are
    deterministic: the results equal those of each job run alone, bit for bit."""
    shapes = [(1500, 1100, 64), (900, 1700, 32)]
    data = []
    for k, (n, m, r) in enumerate(shapes):
        g = np.random.Generator(np.random.PCG64(40 + k))
        V = np.asfortranarray(g.random((n, m), dtype=np.float32))
        W, H = inputs.factors(50 + k, n, m, r)
        data.append((V, W, H))
    alone = []
    for V, W, H in data:
        with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H, eps=1e-9, precision="bf16") as nmf:
            for _ in range(12):
                nmf.DoIteration()
            alone.append((nmf.GetW(), nmf.GetH(), nmf.QualityImprovement()))
    jobs = [gpu.NMF_MultiplicativeEuclidianDistance(V, W, H, eps=1e-9, precision="bf16") for V, W, H in data]
    try:
        for _ in range(12):
            for nmf in jobs:
                nmf.DoIteration()
        for nmf, (Wa, Ha, qa) in zip(jobs, alone):
            assert np.array_equal(nmf.GetW(), Wa) and np.array_equal(nmf.GetH(), Ha)
            assert nmf.QualityImprovement() == qa
    finally:
        for nmf in jobs:
            nmf.close()


def test_pool_reuse_and_trim(gpu):
    """Jobs take device memory from the library's pool: a job made after another was destroyed reuses
    it, after trim_pool it is allocated afresh; the results do not depend on either."""
    n, m, r = 1200, 900, 64
    V = inputs.uniform_matrix(81, n, m)
    W, H = inputs.factors(82, n, m, r)
    outs = []
    for trim in (False, False, True):
        if trim:
            gpu.trim_pool()
        with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H, eps=1e-9, precision="bf16", quality_interval=0) as nmf:
            nmf.Iterate(4)
            outs.append((nmf.GetW(), nmf.GetH()))
    for Wk, Hk in outs[1:]:
        assert np.array_equal(Wk, outs[0][0]) and np.array_equal(Hk, outs[0][1])


def _slice_index(total, seed, edge=256, inner=256):
    """Rows (or columns) to check: the first and last `edge`, and `inner` drawn from the rest (sorted),
    so whole 128-row tiles at both ends and tiles split between stream-K segments are covered."""
    g = np.random.Generator(np.random.PCG64(seed))
    mid = np.sort(g.choice(np.arange(edge, total - edge), size=inner, replace=False))
    return np.r_[np.arange(edge), mid, np.arange(total - edge, total)]


def test_headline_shape_one_iteration_matches_emulation(gpu):
    """The benchmark workload itself (V 8192 x 8192 = A B + |N(0,0.01)|, r = 64, eps 1e-9): one BF16
    iteration (two launches of the fused half-step kernel) against the exact emulation, evaluated on
    768 columns of H and 768 rows of W -- the emulated FP64 products of the whole matrices would take
    minutes on the host.  Same bound as the other shapes: 2e-5 relative Frobenius."""
    cfg = inputs.large_euclidean(8192, 8192, 64)
    V, W, H, eps = cfg["V"], cfg["W"], cfg["H"], np.float32(cfg["eps"])
    with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H, eps=eps, precision="bf16", quality_interval=0) as nmf:
        nmf.DoIteration()
        W1g, H1g = nmf.GetW(), nmf.GetH()
    e = float(eps)
    cols = _slice_index(8192, 1)
    rows = _slice_index(8192, 2)
    Wb = bf16(W)
    Wd, Hd = W.astype(np.float64), H.astype(np.float64)
    H1 = Hd[:, cols] * (Wb.T @ bf16(V[:, cols])) / ((Wd.T @ Wd) @ Hd[:, cols] + e)
    assert rel(H1g[:, cols], H1) <= 2e-5, "H-step (fused half-step kernel) differs at 8192^2 r=64"
    Hg = H1g.astype(np.float64)
    W1 = Wd[rows] * (bf16(V[rows, :]) @ bf16(H1g).T) / (Wd[rows] @ (Hg @ Hg.T) + e)
    assert rel(W1g[rows], W1) <= 2e-5, "W-step (fused half-step kernel) differs at 8192^2 r=64"
