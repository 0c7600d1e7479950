"""Serving with continuous batching (over the C ABI): the ``Server`` handle and a trace replayer.

The scheduler itself is native (gpumlib_gb300/csrc/serve.cu): it admits jobs
into stream slots as slots and HBM budget free up, advances admitted jobs in
chunks of iterations with asynchronous FP64 residual checks, and retires them
at residual <= tol or max_iters.  ``replay`` submits a trace's jobs at their
arrival times from a host thread and collects the results.
"""
import ctypes
import threading
import time

import numpy as np

from . import _native


class ServerResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_longlong), ("rule", ctypes.c_int), ("n", ctypes.c_int), ("m", ctypes.c_int),
                ("r", ctypes.c_int), ("iters", ctypes.c_int), ("precision", ctypes.c_int),
                ("status", ctypes.c_int), ("residual", ctypes.c_double), ("t_submit", ctypes.c_double),
                ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


PRECISIONS = {"fp32": 0, "bf16": 1}


class Server:
    def __init__(self, slots=64, hbm_budget_gb=150.0, precision="bf16", check_every=10, tol=1e-3, max_iters=500,
                 keep_factors=False, grid_policy=None):
        self._lib = _native.load()
        h = ctypes.c_void_p()
        _native.check(self._lib.gpunmf_server_create(int(slots), int(hbm_budget_gb * (1 << 30)),
                                                     PRECISIONS[precision], int(check_every), float(tol),
                                                     int(max_iters), 1 if keep_factors else 0, ctypes.byref(h)))
        self._h = h
        self.keep = keep_factors
        if grid_policy is not None:   # (blocks per CTA, max CTAs per job); see gpunmf_server_set_grid_policy
            _native.check(self._lib.gpunmf_server_set_grid_policy(self._h, int(grid_policy[0]), int(grid_policy[1])))

    def submit(self, job_id, rule, n, m, r, seed, eps=1e-9):
        _native.check(self._lib.gpunmf_server_submit(self._h, int(job_id), int(rule), int(n), int(m), int(r),
                                                     int(seed), float(eps)))

    def poll(self, cap=4096):
        buf = (ServerResult * cap)()
        k = self._lib.gpunmf_server_poll(self._h, buf, cap)
        return [buf[i].as_dict() for i in range(k)]

    def fetch(self, job_id, n, m, r):
        res = ServerResult()
        W = np.empty((n, r), dtype=np.float32, order="F")
        H = np.empty((r, m), dtype=np.float32, order="F")
        _native.check(self._lib.gpunmf_server_fetch(self._h, int(job_id), ctypes.byref(res),
                                                    W.ctypes.data_as(ctypes.c_void_p),
                                                    H.ctypes.data_as(ctypes.c_void_p)))
        return res.as_dict(), W, H

    def drain(self, timeout_s=600.0):
        st = self._lib.gpunmf_server_drain(self._h, float(timeout_s))
        return st == 0

    def stats(self):
        sub, fin = ctypes.c_longlong(), ctypes.c_longlong()
        pend, act = ctypes.c_int(), ctypes.c_int()
        used = ctypes.c_size_t()
        _native.check(self._lib.gpunmf_server_stats(self._h, ctypes.byref(sub), ctypes.byref(fin),
                                                    ctypes.byref(pend), ctypes.byref(act), ctypes.byref(used)))
        return {"submitted": sub.value, "finished": fin.value, "pending": pend.value, "active": act.value,
                "bytes_in_use": used.value}

    def clock(self):
        return self._lib.gpunmf_server_clock(self._h)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gpunmf_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def replay(server, trace, drain_timeout_s=120.0, eps=1e-9):
    """Submit each job of `trace` at its arrival time `t` (seconds) and wait for the results.

    Returns (results, makespan_s, unfinished) where unfinished lists the jobs still
    pending or running when the drain timed out (with their submit times)."""
    t_start = server.clock()
    submitted = {}

    def feeder():
        for job in trace:
            delay = job["t"] - (server.clock() - t_start)
            if delay > 0:
                time.sleep(delay)
            server.submit(job["id"], job["rule"], job["n"], job["m"], job["r"], job["seed"], eps)
            submitted[job["id"]] = server.clock()

    th = threading.Thread(target=feeder, daemon=True)
    th.start()
    results = []
    deadline = None
    while True:
        results.extend(server.poll())
        if not th.is_alive():
            if deadline is None:
                deadline = time.perf_counter() + drain_timeout_s
            st = server.stats()
            if st["finished"] >= st["submitted"] and len(results) >= len(trace):
                break
            if time.perf_counter() > deadline:
                break
        time.sleep(0.005)
    results.extend(server.poll())
    makespan = server.clock() - t_start
    done_ids = {r["id"] for r in results}
    unfinished = [{"id": i, "t_submit": t} for i, t in submitted.items() if i not in done_ids]
    return results, makespan, unfinished


def latency_summary(results, unfinished, now):
    """p50 / p99 latency (s) over finished jobs; unfinished jobs count with their age so far (a lower bound)."""
    lat = [r["t_done"] - r["t_submit"] for r in results if r["status"] == 0]
    lat += [now - u["t_submit"] for u in unfinished]
    if not lat:
        return {"p50_s": None, "p99_s": None}
    a = np.array(lat)
    return {"p50_s": float(np.percentile(a, 50)), "p99_s": float(np.percentile(a, 99)),
            "mean_s": float(a.mean()), "max_s": float(a.max())}
