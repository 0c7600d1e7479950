"""Parity of the plain FP32 path (the drop-in) with the reference.

Bar (from the engine's contract): after the same iterations from the same
seeded inputs, W H agrees with the reference's own implementation within
1e-4 relative Frobenius; W and H individually within 1e-4 as well.  The
reference outputs are the golden vectors of its HostNMF
(tests/golden/hostnmf_golden.npz); larger shapes compare with the oracle.
"""
import numpy as np
import pytest

import oracle
from conftest import rel
from golden.make_golden import CASES, case_inputs
from gpumlib_gb300 import inputs

pytestmark = pytest.mark.gpu

TOL_WH = 1e-4
TOL_FACTOR = 1e-4


def run_gpu(g, rule, V, W, H, iters, updateW=True, eps=1e-8, precision="fp32", **kw):
    """Rule numbers as in gpunmf_rule: 0/1 multiplicative, 2/3 additive (both factors), 4 fixed-H."""
    with g.make(rule, V, W, H, eps=eps, precision=precision, **kw) as nmf:
        nmf.Iterate(iters, updateW)
        return nmf.GetW(), nmf.GetH(), nmf.Residual()


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_fp32_matches_reference_golden(gpu, golden, case):
    data, _ = golden
    name, rule, n, m, r, iters, updateW = case[:7]
    V, W, H = case_inputs(case)
    Wg, Hg, _ = run_gpu(gpu, rule, V, W, H, iters, updateW)
    Wr, Hr = data[name + "/W"], data[name + "/H"]
    assert rel(Wg.astype(np.float64) @ Hg, Wr.astype(np.float64) @ Hr) <= TOL_WH
    assert rel(Wg, Wr) <= TOL_FACTOR
    assert rel(Hg, Hr) <= TOL_FACTOR
    assert np.all(Wg >= 0) and np.all(Hg >= 0)


def test_fp32_residual_trajectory_matches_reference(gpu, golden):
    data, _ = golden
    case = [c for c in CASES if c[0] == "me_1024x512_r16"][0]
    name, rule, n, m, r, iters, updateW = case[:7]
    V, W, H = case_inputs(case)
    ref = data[name + "/resid"]
    with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H) as nmf:
        got = []
        for _ in range(iters):
            nmf.DoIteration()
            got.append(nmf.Residual())
    np.testing.assert_allclose(got, ref, rtol=1e-5)


def test_plain_euclidean_workload_eps_1e9(gpu):
    """The 1024x512, r=16, 200-iteration workload with eps 1e-9, against the oracle at eps 1e-9."""
    cfg = inputs.plain_euclidean_1024x512()
    Wg, Hg, res = run_gpu(gpu, 0, cfg["V"], cfg["W"], cfg["H"], cfg["iters"], eps=cfg["eps"])
    Wo, Ho = oracle.hostnmf_run(0, cfg["V"], cfg["W"], cfg["H"], cfg["iters"], eps=np.float32(1e-9), nthreads=8)
    assert rel(Wg.astype(np.float64) @ Hg, Wo.astype(np.float64) @ Ho) <= TOL_WH
    assert abs(res - oracle.residual(cfg["V"], Wo, Ho, 8)) <= 1e-5


@pytest.mark.parametrize("rule", [0, 1])
@pytest.mark.parametrize("shape", [(129, 257, 65), (1, 1, 1), (1, 300, 2), (300, 1, 3), (257, 96, 128),
                                   (1500, 700, 40)])
def test_fp32_odd_shapes_vs_f64_oracle(gpu, rule, shape):
    n, m, r = shape
    iters = 8
    V = inputs.uniform_matrix(31 + n, n, m)
    W, H = inputs.factors(37 + m, n, m, r)
    Wg, Hg, _ = run_gpu(gpu, rule, V, W, H, iters)
    Wd, Hd = oracle.f64_run(rule, V, W, H, iters, nthreads=8)
    assert rel(Wg.astype(np.float64) @ Hg, Wd @ Hd) <= TOL_WH


def test_fp32_deterministic(gpu):
    n, m, r = 700, 500, 24
    V = inputs.uniform_matrix(3, n, m)
    W, H = inputs.factors(4, n, m, r)
    for rule in (0, 1):
        a = run_gpu(gpu, rule, V, W, H, 5)
        b = run_gpu(gpu, rule, V, W, H, 5)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_euclidean_objective_non_increasing(gpu):
    """Lee-Seung: the Euclidean MU never increases ||V - WH|| (up to rounding)."""
    V = inputs.lowrank_gamma(2048, 1536, 32, 2.0, 0.5, seed=9)
    W, H = inputs.factors(10, 2048, 1536, 32)
    with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H, eps=1e-9) as nmf:
        prev = nmf.Residual()
        for _ in range(25):
            nmf.DoIteration()
            cur = nmf.Residual()
            assert cur <= prev * (1 + 1e-6)
            prev = cur


def test_kl_objective_non_increasing(gpu):
    n, m, r = 1024, 768, 16
    g = np.random.Generator(np.random.PCG64(11))
    V = np.asfortranarray(g.poisson(3.0, size=(n, m)).astype(np.float32))
    W, H = inputs.factors(12, n, m, r)
    with gpu.NMF_MultiplicativeDivergence(V, W, H, eps=1e-9) as nmf:
        prev = nmf.ObjectiveKL()
        for _ in range(15):
            nmf.DoIteration()
            cur = nmf.ObjectiveKL()
            assert cur <= prev * (1 + 1e-6) + 1e-6
            prev = cur


def test_exact_factorisation_converges(gpu):
    n, m, r = 512, 384, 8
    W0, H0 = inputs.factors(13, n, m, r, add=0.05)
    V = np.asfortranarray((W0.astype(np.float64) @ H0).astype(np.float32))
    W, H = inputs.factors(14, n, m, r)
    with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H) as nmf:
        r0 = nmf.Residual()
        nmf.Iterate(400)
        r1 = nmf.Residual()
    assert r1 < 0.1 * r0 and r1 < 0.05


def test_update_w_false_keeps_w(gpu):
    n, m, r = 200, 150, 5
    V = inputs.uniform_matrix(15, n, m)
    W, H = inputs.factors(16, n, m, r)
    for rule in (0, 1):
        Wg, Hg, _ = run_gpu(gpu, rule, V, W, H, 4, updateW=False)
        assert np.array_equal(Wg, W)
        _, Ho = oracle.hostnmf_run(rule, V, W, H, 4, updateW=False, eps=1e-8)
        assert rel(Hg, Ho) <= TOL_FACTOR


def test_random_constructor_uses_counter_generator(gpu):
    n, m, r = 64, 48, 3
    V = inputs.uniform_matrix(17, n, m)
    with gpu.NMF_MultiplicativeEuclidianDistance(V, r, seed=99) as nmf:
        W = nmf.GetW()
        H = nmf.GetH()
    eps = np.float32(1e-8)
    assert np.array_equal(W, inputs.uniform_matrix(99, n, r) + eps)
    assert np.array_equal(H, inputs.uniform_matrix(99, r, m, offset=n * r) + eps)


def test_getwh_matches_factors(gpu):
    n, m, r = 333, 222, 11
    V = inputs.uniform_matrix(18, n, m)
    W, H = inputs.factors(19, n, m, r)
    with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H) as nmf:
        nmf.Iterate(3)
        WH = nmf.GetWH()
        Wg, Hg = nmf.GetW(), nmf.GetH()
    assert rel(WH, Wg.astype(np.float64) @ Hg) <= 1e-6
