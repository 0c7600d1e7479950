"""The CPU oracle against golden vectors made by the reference's own HostNMF.

The golden file holds W, H and per-iteration residuals produced by
src/examples/FacesNMF/HostNMF.h compiled from the reference sources
(tests/golden/make_golden.py).  The float transcription in
oracle/nmf_oracle.c must reproduce them bit for bit.
"""
import numpy as np
import pytest

import oracle
from golden.make_golden import CASES, case_inputs


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_reference_bits(case, golden):
    data, _ = golden
    name, rule, n, m, r, iters, updateW = case[:7]
    V, W, H = case_inputs(case)
    Wo, Ho = oracle.hostnmf_run(rule, V, W, H, iters, updateW=updateW, eps=1e-8, nthreads=2)
    assert np.array_equal(Wo, data[name + "/W"]), "W differs from the reference"
    assert np.array_equal(Ho, data[name + "/H"]), "H differs from the reference"


def test_oracle_residual_trajectory(golden):
    data, _ = golden
    case = [c for c in CASES if c[0] == "me_1024x512_r16"][0]
    name, rule, n, m, r, iters, updateW = case[:7]
    V, W, H = case_inputs(case)
    _, _, res = oracle.hostnmf_run(rule, V, W, H, 20, updateW=updateW, eps=1e-8, nthreads=4,
                                   residuals=True)
    np.testing.assert_allclose(res, data[name + "/resid"][:20], rtol=1e-12)


def test_oracle_thread_count_invariant():
    from gpumlib_gb300 import inputs
    V = inputs.uniform_matrix(5, 70, 45)
    W, H = inputs.factors(6, 70, 45, 4)
    for rule in (0, 1, 2, 3):
        a = oracle.hostnmf_run(rule, V, W, H, 5, nthreads=1)
        b = oracle.hostnmf_run(rule, V, W, H, 5, nthreads=7)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_oracle_fixed_h_additive():
    """skip_h reproduces the reference GPU class's additive Euclidean H step, which leaves H as it
    was (nmf_additive_euclidian.cpp:37-42); its W step is HostNMF's (HostNMF.h:176-189)."""
    from gpumlib_gb300 import inputs
    V = inputs.uniform_matrix(7, 60, 40)
    W, H = inputs.factors(8, 60, 40, 5)
    Wf, Hf = oracle.hostnmf_run(2, V, W, H, 3, skip_h=True)
    assert np.array_equal(Hf, H)
    # one W step from the same H equals the full rule's W step when H is not updated first
    W1, H1 = oracle.hostnmf_run(2, V, W, H, 1, skip_h=True)
    Wd, Hd = W.astype(np.float64), H.astype(np.float64)
    exp = np.maximum(Wd + Wd / (Wd @ (Hd @ Hd.T)) * (V @ Hd.T - Wd @ (Hd @ Hd.T)), 0)
    assert np.linalg.norm(W1 - exp) / np.linalg.norm(exp) < 1e-5


def test_f64_oracle_close_to_float_reference(golden):
    """The FP64 statement of the GPU rules agrees with the float reference to rounding."""
    data, _ = golden
    for nm in ("me_odd_37x23_r3", "kl_odd_33x17_r5"):
        case = [c for c in CASES if c[0] == nm][0]
        name, rule, n, m, r, iters, updateW = case[:7]
        V, W, H = case_inputs(case)
        Wd, Hd = oracle.f64_run(rule, V, W, H, iters, updateW=updateW, eps=1e-8)
        WHd = Wd @ Hd
        WHg = data[name + "/W"].astype(np.float64) @ data[name + "/H"]
        assert np.linalg.norm(WHd - WHg) / np.linalg.norm(WHd) < 1e-5


def test_quality_formula():
    V = np.array([[1.0, 2.0], [0.0, 3.0]], dtype=np.float32, order="F")
    WH = np.array([[0.5, 1.0], [2.0, 4.0]], dtype=np.float32, order="F")
    q = oracle.quality(V, WH, eps=1e-8)
    exp = sum(float(v) * np.log10(float(w) + 1e-8) - float(w) for v, w in zip(V.ravel(), WH.ravel()))
    assert abs(q - exp) < 1e-5


def test_planted_error_is_caught(golden):
    """A mistake planted in the oracle's inputs must break bit-equality (the check has teeth)."""
    data, _ = golden
    case = [c for c in CASES if c[0] == "me_odd_37x23_r3"][0]
    name, rule, n, m, r, iters, updateW = case[:7]
    V, W, H = case_inputs(case)
    V = V.copy(order="F")
    V[5, 7] = np.nextafter(V[5, 7], np.float32(2.0))
    Wo, Ho = oracle.hostnmf_run(rule, V, W, H, iters, updateW=updateW, eps=1e-8)
    assert not np.array_equal(Wo, data[name + "/W"])


def test_oracle_grouped_layout_and_stop():
    """TrainUsingGroups restated: block layout and the lagged stopping test."""
    from gpumlib_gb300 import inputs
    V = inputs.uniform_matrix(21, 30, 47)
    W, H = inputs.factors(22, 30, 47, 7)
    Wo, Ho, its, deltas = oracle.grouped_run(1, V, W, H, 15, 0.5, 400)
    assert len(its) == 3                      # 47 // 15 blocks, rank 7 // 3 = 2 each
    assert np.array_equal(Wo[:, 6:], W[:, 6:]) and np.array_equal(Ho[:, 45:], H[:, 45:])
    for s in range(3):
        block = Ho[:, s * 15:(s + 1) * 15]
        assert np.all(np.delete(block, np.s_[2 * s:2 * s + 2], axis=0) == 0)
        d = deltas[s]
        assert d[0] == 1.0 and d[1] == 1.0    # no improvement before the third sample
        assert its[s] == len(d) and (d[-1] < 0.5 or its[s] == 400)
        assert all(x >= 0.5 for x in d[2:-1] if x != 1.0)


def test_f64_blas_restatement_matches_f64_loops():
    """The BLAS-backed FP64 rules (used for full-size error checks) agree with the FP64 loops."""
    from gpumlib_gb300 import inputs
    for rule, (n, m, r) in ((0, (130, 97, 9)), (1, (61, 150, 5))):
        V = inputs.uniform_matrix(31 + rule, n, m, add=0.01)
        W, H = inputs.factors(41 + rule, n, m, r)
        for updateW in (True, False):
            Wa, Ha = oracle.f64_run(rule, V, W, H, 4, updateW=updateW, eps=1e-9)
            Wb, Hb = oracle.f64_run_blas(rule, V, W, H, 4, updateW=updateW, eps=1e-9)
            err = oracle.factor_errors(Wb, Hb, Wa, Ha)
            assert max(err.values()) < 1e-12, (rule, updateW, err)
