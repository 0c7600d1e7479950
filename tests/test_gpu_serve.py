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
