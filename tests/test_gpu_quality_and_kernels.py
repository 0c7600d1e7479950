"""Quality bookkeeping (nmf_base.h:70-89) and the kernel-level entry points
(nmf_kernels.h:44-142) against the oracle."""
import ctypes

import numpy as np
import pytest

import oracle
from gpumlib_gb300 import _native, inputs

pytestmark = pytest.mark.gpu


class QualityModel:
    """Restatement of NMF::DetermineQualityImprovement with every read-back complete."""

    def __init__(self):
        self.times = 0
        self.last = -1.0
        self.delta = 1.0
        self.value = 0.0   # vquality initial value (nmf_base.h:97)

    def sample(self, new_value):
        q = self.value
        if self.times > 2:
            self.delta = q - self.last
        self.times += 1
        if self.times <= 3:
            self.times += 1
        self.last = q
        self.value = new_value


def test_model_matches_reference_counting():
    m = QualityModel()
    deltas = []
    for k in range(6):
        m.sample(float(10 * (k + 1)))
        deltas.append(m.delta)
    # samples 1 and 2 keep the initial 1.0; the third compares q(start of it 2) with q(start of it 1)
    assert deltas[:2] == [1.0, 1.0] and deltas[2] == 10.0


@pytest.mark.parametrize("rule", [0, 1])
def test_quality_improvement_sequence(gpu, rule):
    n, m, r = 300, 200, 6
    V = inputs.uniform_matrix(41, n, m)
    W, H = inputs.factors(42, n, m, r)
    cls = gpu.NMF_MultiplicativeEuclidianDistance if rule == 0 else gpu.NMF_MultiplicativeDivergence
    model = QualityModel()
    Wc, Hc = W.copy(order="F"), H.copy(order="F")
    with cls(V, W, H) as nmf:
        for it in range(7):
            # the quality of this iteration is evaluated on the factors it starts from
            q_now = oracle.quality(V, oracle.hostnmf_wh(Wc, Hc), eps=1e-8)
            model.sample(q_now)
            nmf.DoIteration()
            got = nmf.QualityImprovement()
            scale = max(1.0, abs(q_now))
            assert abs(got - model.delta) <= 2e-5 * scale, (it, got, model.delta)
            Wc, Hc = oracle.hostnmf_run(rule, V, Wc, Hc, 1, eps=1e-8, clamp_sums=True)


def test_quality_interval_zero_disables(gpu):
    V = inputs.uniform_matrix(43, 64, 64)
    W, H = inputs.factors(44, 64, 64, 4)
    with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H, quality_interval=0) as nmf:
        nmf.Iterate(10)
        assert nmf.QualityImprovement() == 1.0


@pytest.mark.parametrize("precision,rule", [("fp32", 0), ("fp32", 1), ("bf16", 0), ("bf16", 1)])
def test_when_ready_with_every_readback_complete_matches_interval_one(gpu, precision, rule):
    """QUALITY_WHEN_READY (the reference's rule, nmf_base.h:71) samples an iteration only when the
    previous sample's read-back is complete.  With the host waiting for the job after every iteration
    every read-back is complete, so it samples every iteration: the same improvements as interval 1
    and the same factors, bit for bit (sampling never changes the factors)."""
    n, m, r = 1024, 768, 64
    V = inputs.lowrank_gamma(n, m, 16, 2.0, 0.5, seed=45)
    W, H = inputs.factors(46, n, m, r)
    runs = []
    for k in (1, gpu.QUALITY_WHEN_READY):
        with gpu.make(rule, V, W, H, eps=1e-9, precision=precision, quality_interval=k) as nmf:
            d = []
            for _ in range(8):
                nmf.DoIteration()
                nmf.GetH()   # waits for the job's stream
                d.append(nmf.QualityImprovement())
            runs.append((d, nmf.GetW(), nmf.GetH()))
    (d1, W1, H1), (d2, W2, H2) = runs
    assert d1 == d2 and d1[2] != 1.0
    assert np.array_equal(W1, W2) and np.array_equal(H1, H2)


@pytest.mark.parametrize("rule", [0, 1])
def test_when_ready_without_waits_keeps_factors(gpu, rule):
    """Under QUALITY_WHEN_READY with no host waits the iterations that sample depend on timing, but
    the factors do not: 60 BF16 iterations end with the W and H of a job that never samples, bit for
    bit, and the improvement read is finite."""
    n, m, r = 2048, 1536, 64
    V = inputs.lowrank_gamma(n, m, 16, 2.0, 0.5, seed=47)
    W, H = inputs.factors(48, n, m, r)
    out = []
    for k in (0, gpu.QUALITY_WHEN_READY):
        with gpu.make(rule, V, W, H, eps=1e-9, precision="bf16", quality_interval=k) as nmf:
            for _ in range(60):
                nmf.DoIteration()
                q = nmf.QualityImprovement()
            out.append((nmf.GetW(), nmf.GetH(), q))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == 1.0 and np.isfinite(out[1][2])


# ---------------------------------------------------------------------------
# kernel API on device buffers (torch used only to hold device memory)
# ---------------------------------------------------------------------------
torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float32).ravel(order="F"))).cuda()


def ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_euclidean_update_entry_point(gpu):
    lib = _native.load()
    g = np.random.Generator(np.random.PCG64(1))
    count = 10007
    nm, dm, x = (g.random(count, dtype=np.float32) for _ in range(3))
    tn, td, tx = dev(nm), dev(dm), dev(x)
    assert lib.gpumlib_cuda_nmf_multiplicative_euclidean_update_matrix(20, 512, ptr(tn), ptr(td), ptr(tx), count) == 0
    torch.cuda.synchronize()
    exp = x * (nm / (dm + np.float32(1e-8)))
    np.testing.assert_allclose(tx.cpu().numpy(), exp, rtol=1e-6)


def test_sum_entry_points(gpu):
    lib = _native.load()
    n, m, r = 517, 333, 9
    W, H = inputs.factors(5, n, m, r)
    W[:, 3] = 0.0
    H[4, :] = 0.0
    tw, th, ts = dev(W), dev(H), torch.zeros(r, device="cuda")
    assert lib.gpumlib_nmf_sum_w(512, ptr(tw), n, r, ptr(ts)) == 0
    torch.cuda.synchronize()
    exp = np.maximum(W.astype(np.float64).sum(axis=0), 1e-8)
    np.testing.assert_allclose(ts.cpu().numpy(), exp, rtol=1e-5)
    assert lib.gpumlib_nmf_sum_h(512, ptr(th), r, m, ptr(ts)) == 0
    torch.cuda.synchronize()
    exp = np.maximum(H.astype(np.float64).sum(axis=1), 1e-8)
    np.testing.assert_allclose(ts.cpu().numpy(), exp, rtol=1e-5)


def test_quality_entry_point(gpu):
    lib = _native.load()
    n, m, r = 411, 205, 7
    V = inputs.uniform_matrix(6, n, m)
    W, H = inputs.factors(7, n, m, r)
    WH = oracle.hostnmf_wh(W, H)
    tv, twh, tq = dev(V), dev(WH), torch.zeros(1, device="cuda")
    assert lib.gpumlib_nmf_quality(512, ptr(tv), ptr(twh), n * m, ptr(tq)) == 0
    torch.cuda.synchronize()
    exp = oracle.quality(V, WH, eps=1e-8)
    assert abs(tq.item() - exp) <= 1e-5 * abs(exp)


@pytest.mark.parametrize("which", ["h", "w"])
def test_kl_update_entry_points(gpu, which):
    lib = _native.load()
    n, m, r = 301, 203, 13
    V = inputs.uniform_matrix(8, n, m)
    W, H = inputs.factors(9, n, m, r)
    WH = oracle.hostnmf_wh(W, H)
    tv, tw, th, twh = dev(V), dev(W), dev(H), dev(WH)
    Vd, Wd, Hd = (a.astype(np.float64) for a in (V, W, H))
    R = Vd / (WH.astype(np.float64) + 1e-8)
    d3 = _native.Dim3(1, 1, 1)
    if which == "h":
        sums = np.maximum(Wd.sum(axis=0), 1e-8).astype(np.float32)
        ts = dev(sums)
        assert lib.gpumlib_cuda_nmf_multiplicative_divergence_update_matrix_h(
            d3, d3, ptr(th), ptr(tw), ptr(tv), ptr(twh), ptr(ts), n, m, r) == 0
        torch.cuda.synchronize()
        got = th.cpu().numpy().reshape(m, r).T
        exp = Hd * (Wd.T @ R) / sums[:, None]
    else:
        sums = np.maximum(Hd.sum(axis=1), 1e-8).astype(np.float32)
        ts = dev(sums)
        assert lib.gpumlib_cuda_nmf_multiplicative_divergence_update_matrix_w(
            d3, d3, ptr(tw), ptr(th), ptr(tv), ptr(twh), ptr(ts), n, m, r) == 0
        torch.cuda.synchronize()
        got = tw.cpu().numpy().reshape(r, n).T
        exp = Wd * (R @ Hd.T) / sums[None, :]
    np.testing.assert_allclose(got, exp, rtol=2e-5)


def test_status_errors_on_gpu(gpu):
    lib = _native.load()
    V = inputs.uniform_matrix(1, 16, 8)
    with gpu.NMF_MultiplicativeEuclidianDistance(V, 2) as nmf:
        assert lib.gpunmf_set_quality_interval(nmf._h, -2) == 1
        assert lib.gpunmf_iterate(nmf._h, -3, 1) == 1
    with pytest.raises(ValueError):
        gpu.NMF_MultiplicativeEuclidianDistance(V, np.ones((15, 2), np.float32), np.ones((2, 8), np.float32))
