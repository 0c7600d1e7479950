"""Serving with continuous batching: admission, overlap, stop criteria, and
"the same result alone and in the mix" (bound: 1e-6 relative on W and H,
identical iteration counts; the kernels are deterministic, so in practice the
results are bit-identical)."""
import time

import numpy as np
import pytest

from conftest import rel
from gpumlib_gb300 import serve

pytestmark = pytest.mark.gpu

TOL_MIX = 1e-6


def run_alone(job, precision):
    with serve.Server(slots=4, precision=precision, check_every=10, max_iters=120, keep_factors=True) as s:
        s.submit(job["id"], job["rule"], job["n"], job["m"], job["r"], job["seed"])
        assert s.drain(120)
        return s.fetch(job["id"], job["n"], job["m"], job["r"])


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_result_alone_equals_result_in_mix(gpu, precision):
    targets = [dict(id=1, rule=0, n=700, m=500, r=24, seed=11), dict(id=2, rule=1, n=300, m=900, r=12, seed=12),
               dict(id=3, rule=0, n=2000, m=1500, r=64, seed=13)]
    alone = {j["id"]: run_alone(j, precision) for j in targets}
    g = np.random.Generator(np.random.PCG64(5))
    others = [dict(id=100 + k, rule=int(g.random() < 0.3), n=int(g.integers(64, 1500)), m=int(g.integers(64, 1500)),
                   r=int(g.integers(8, 65)), seed=1000 + k) for k in range(24)]
    mix = others[:8] + [targets[0]] + others[8:16] + [targets[1]] + others[16:] + [targets[2]]
    with serve.Server(slots=16, precision=precision, check_every=10, max_iters=120, keep_factors=True) as s:
        for j in mix:
            s.submit(j["id"], j["rule"], j["n"], j["m"], j["r"], j["seed"])
        assert s.drain(300)
        for j in targets:
            res, W, H = s.fetch(j["id"], j["n"], j["m"], j["r"])
            ares, aW, aH = alone[j["id"]]
            assert res["status"] == 0 and ares["status"] == 0
            assert res["iters"] == ares["iters"]
            assert rel(W, aW) <= TOL_MIX and rel(H, aH) <= TOL_MIX
            assert abs(res["residual"] - ares["residual"]) <= TOL_MIX * max(1.0, ares["residual"])
        # the mix really overlapped: some job was admitted before an earlier one finished
        rs = [s.fetch(j["id"], j["n"], j["m"], j["r"])[0] for j in mix]
        rs.sort(key=lambda x: x["t_admit"])
        assert any(rs[k + 1]["t_admit"] < rs[k]["t_done"] for k in range(len(rs) - 1))


def test_grid_policy_changes_no_result_beyond_rounding(gpu):
    """The server's per-job CTA cap (gpunmf_server_set_grid_policy) changes only the kernels' stream-K
    partition, hence FP32 summation orders: same iterations, residuals within 1e-4 relative."""
    jobs = [dict(id=1, rule=0, n=1500, m=1300, r=48, seed=31), dict(id=2, rule=1, n=900, m=1100, r=32, seed=32)]
    out = {}
    for pol in ((0, 0), (1, 5)):
        with serve.Server(slots=4, precision="bf16", check_every=10, max_iters=40, keep_factors=True,
                          grid_policy=pol) as s:
            for j in jobs:
                s.submit(j["id"], j["rule"], j["n"], j["m"], j["r"], j["seed"])
            assert s.drain(120)
            out[pol] = [s.fetch(j["id"], j["n"], j["m"], j["r"]) for j in jobs]
    for (ra, Wa, Ha), (rb, Wb, Hb) in zip(out[(0, 0)], out[(1, 5)]):
        assert ra["status"] == 0 and rb["status"] == 0 and ra["iters"] == rb["iters"]
        assert abs(ra["residual"] - rb["residual"]) <= 1e-4 * ra["residual"]
        assert rel(Wb.astype(np.float64) @ Hb, Wa.astype(np.float64) @ Ha) <= 5e-3


def test_admission_respects_hbm_budget(gpu):
    from gpumlib_gb300 import nmf
    jobs = [dict(id=k, rule=0, n=1024, m=1024, r=32, seed=50 + k) for k in range(6)]
    one = nmf.footprint_bytes(0, 1024, 1024, 32, "fp32")
    budget_gb = 1.5 * one / (1 << 30)  # room for one job at a time
    with serve.Server(slots=8, hbm_budget_gb=budget_gb, precision="fp32", check_every=10, max_iters=30,
                      keep_factors=True) as s:
        for j in jobs:
            s.submit(j["id"], j["rule"], j["n"], j["m"], j["r"], j["seed"])
        assert s.drain(120)
        rs = sorted((s.fetch(j["id"], 1024, 1024, 32)[0] for j in jobs), key=lambda x: x["t_admit"])
    assert all(r["status"] == 0 for r in rs)
    for a, b in zip(rs, rs[1:]):
        assert b["t_admit"] >= a["t_done"] - 1e-6, "two jobs were resident beyond the budget"


def test_oversized_job_is_rejected(gpu):
    with serve.Server(slots=2, hbm_budget_gb=0.01, precision="fp32", keep_factors=True) as s:
        s.submit(7, 0, 4096, 4096, 64, 1)
        assert s.drain(30)
        res, _, _ = s.fetch(7, 4096, 4096, 64)
    assert res["status"] == 7  # GPUNMF_ERR_REJECTED


def test_stop_criteria(gpu):
    # a reachable tolerance: the job retires early, at a check that met it
    with serve.Server(slots=4, precision="bf16", check_every=10, tol=0.05, max_iters=200) as s:
        s.submit(1, 0, 512, 512, 64, 21)
        assert s.drain(120)
        res = s.poll()
    # a tolerance the data cannot reach (noise floor): the job stops at max_iters
    with serve.Server(slots=4, precision="bf16", check_every=10, tol=1e-9, max_iters=50) as s2:
        s2.submit(2, 0, 512, 512, 64, 21)
        assert s2.drain(120)
        res2 = s2.poll()
    assert res[0]["status"] == 0 and res[0]["residual"] <= 0.05 and res[0]["iters"] < 200
    assert res2[0]["iters"] == 50 and res2[0]["residual"] > 1e-9


def test_replay_trace_small(gpu):
    from gpumlib_gb300 import inputs
    trace = inputs.serving_trace(rate=200.0, duration=0.5, seed=3, lo=64, hi=512, rmin=8, rmax=16)
    with serve.Server(slots=32, precision="bf16", check_every=10, tol=1e-3, max_iters=100) as s:
        results, makespan, unfinished = serve.replay(s, trace, drain_timeout_s=60)
    assert not unfinished and len(results) == len(trace)
    assert all(r["status"] == 0 for r in results)
    lat = serve.latency_summary(results, unfinished, makespan)
    assert lat["p99_s"] is not None and lat["p99_s"] >= lat["p50_s"] > 0


def _served_inputs(lib, n, m, r, seed):
    """The inputs a served job with this seed starts from, written by the server's own device code."""
    import ctypes
    torch = pytest.importorskip("torch")
    from gpumlib_gb300 import _native, inputs
    dV = torch.empty(n * m, dtype=torch.float32, device="cuda")
    dW = torch.empty(n * r, dtype=torch.float32, device="cuda")
    dH = torch.empty(r * m, dtype=torch.float32, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    _native.check(lib.gpunmf_server_generate(n, m, r, seed, 0.01, p(dV), p(dW), p(dH), None))
    torch.cuda.synchronize()
    return (inputs.colmajor(dV.cpu().numpy(), n, m), inputs.colmajor(dW.cpu().numpy(), n, r),
            inputs.colmajor(dH.cpu().numpy(), r, m))


SERVED = [dict(id=1, rule=0, n=600, m=450, r=16, seed=31), dict(id=2, rule=1, n=350, m=700, r=12, seed=32),
          dict(id=3, rule=0, n=1300, m=900, r=48, seed=33), dict(id=4, rule=1, n=900, m=1100, r=40, seed=34)]


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_served_results_match_oracle(gpu, precision):
    """Served jobs (Euclidean and KL, overlapping on the device) against the CPU oracle from the same
    inputs, rebuilt by the server's generator (and checked against its host twin).  FP32: W H within
    1e-4 of the reference HostNMF arithmetic after the served iteration count (the drop-in bound).
    BF16: W H within 5e-3 of the FP64 oracle (the bound of the other BF16 tests).  Each result's
    residual is the oracle's residual of the returned factors."""
    import oracle
    from gpumlib_gb300 import _native, inputs
    lib = _native.load()
    with serve.Server(slots=8, precision=precision, check_every=10, tol=1e-9, max_iters=60, keep_factors=True) as s:
        for j in SERVED:
            s.submit(j["id"], j["rule"], j["n"], j["m"], j["r"], j["seed"], 1e-9)
        assert s.drain(300)
        out = {j["id"]: s.fetch(j["id"], j["n"], j["m"], j["r"]) for j in SERVED}
    for j in SERVED:
        res, W, H = out[j["id"]]
        assert res["status"] == 0 and res["iters"] == 60
        V, W0, H0 = _served_inputs(lib, j["n"], j["m"], j["r"], j["seed"])
        tV, tW, tH = inputs.serving_job_data(j)
        assert np.array_equal(W0, tW) and np.array_equal(H0, tH) and rel(V, tV) <= 1e-6
        if precision == "fp32":
            Wo, Ho = oracle.hostnmf_run(j["rule"], V, W0, H0, res["iters"], eps=np.float32(1e-9), clamp_sums=True,
                                        nthreads=8)
            bound = 1e-4
        else:
            Wo, Ho = oracle.f64_run_blas(j["rule"], V, W0, H0, res["iters"], eps=1e-9)
            bound = 5e-3
        err = oracle.factor_errors(W, H, Wo, Ho)
        assert err["WH"] <= bound, (j, err)
        assert abs(res["residual"] - oracle.residual(V, W, H)) <= 1e-6 * max(1.0, res["residual"])


def test_served_stop_rule_matches_oracle(gpu):
    """The stop rule of the reference's training loop (FacesNMFDlg.cpp:658-681), with the residual as
    the test: a served FP32 job retires at the first check (every 10 iterations) whose residual is at
    or below tol, the check at which the oracle's trajectory first reaches it."""
    import oracle
    from gpumlib_gb300 import _native
    lib = _native.load()
    j = dict(id=9, rule=0, n=500, m=400, r=32, seed=41)
    V, W0, H0 = _served_inputs(lib, j["n"], j["m"], j["r"], j["seed"])
    _, _, traj = oracle.hostnmf_run(0, V, W0, H0, 200, eps=np.float32(1e-9), nthreads=8, residuals=True)
    checks = traj[9::10]
    tol = float(np.sqrt(checks[3] * checks[4]))  # between the 4th and 5th checks: reached at iteration 50
    with serve.Server(slots=2, precision="fp32", check_every=10, tol=tol, max_iters=200, keep_factors=True) as s:
        s.submit(j["id"], j["rule"], j["n"], j["m"], j["r"], j["seed"], 1e-9)
        assert s.drain(120)
        res, W, H = s.fetch(j["id"], j["n"], j["m"], j["r"])
    assert res["status"] == 0 and res["iters"] == 50, (res, checks[:6], tol)
    assert res["residual"] <= tol < checks[3]
