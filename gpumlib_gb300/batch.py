"""Batched small factorisations and their tile autotuner (over the C ABI).

``Batch`` holds thousands of uneven Euclidean instances on the device and
runs all of them in one persistent, graph-captured launch
(gpumlib_gb300/csrc/batch.cu).  ``autotune`` times every tile configuration
of the matching rank class on a sample of each (rank class, size) bucket and
assigns the fastest to every instance of that bucket.
"""
import ctypes
import time

import numpy as np

from . import _native

_P = ctypes.c_void_p


def _lib():
    return _native.load()


def rank_class(r):
    return 4 if r <= 4 else 8 if r <= 8 else 16 if r <= 16 else 32 if r <= 32 else None


def size_class(n, m):
    nm = n * m
    return 0 if nm < 32768 else 1 if nm < 196608 else 2


def configs():
    lib = _lib()
    ranks = (ctypes.c_int * 64)()
    k = lib.gpunmf_batch_configs(ranks, 64)
    return [ranks[i] for i in range(k)]


class Batch:
    def __init__(self, instances, eps=1e-8):
        """instances: sequence of dicts with V (n x m), W (n x r), H (r x m) numpy arrays."""
        lib = _lib()
        self.count = len(instances)
        self.shapes = []
        Vs, Ws, Hs = [], [], []
        for d in instances:
            V = np.asfortranarray(d["V"], dtype=np.float32)
            W = np.asfortranarray(d["W"], dtype=np.float32)
            H = np.asfortranarray(d["H"], dtype=np.float32)
            n, m = V.shape
            r = W.shape[1]
            if W.shape[0] != n or H.shape != (r, m):
                raise ValueError("instance shapes do not agree")
            self.shapes.append((n, m, r))
            Vs.append(V); Ws.append(W); Hs.append(H)
        self._keep = (Vs, Ws, Hs)
        ns = (ctypes.c_int * self.count)(*[s[0] for s in self.shapes])
        ms = (ctypes.c_int * self.count)(*[s[1] for s in self.shapes])
        rs = (ctypes.c_int * self.count)(*[s[2] for s in self.shapes])
        pv = (ctypes.c_void_p * self.count)(*[a.ctypes.data for a in Vs])
        pw = (ctypes.c_void_p * self.count)(*[a.ctypes.data for a in Ws])
        ph = (ctypes.c_void_p * self.count)(*[a.ctypes.data for a in Hs])
        h = ctypes.c_void_p()
        _native.check(lib.gpunmf_batch_create(self.count, ns, ms, rs, pv, pw, ph, float(eps), ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self.cfg = [None] * self.count

    def run(self, iters):
        _native.check(self._lib.gpunmf_batch_run(self._h, int(iters)))

    def synchronize(self):
        _native.check(self._lib.gpunmf_batch_synchronize(self._h))

    def time(self, iters):
        ms = ctypes.c_float()
        _native.check(self._lib.gpunmf_batch_time(self._h, int(iters), ctypes.byref(ms)))
        return ms.value

    def get(self, k):
        n, m, r = self.shapes[k]
        W = np.empty((n, r), dtype=np.float32, order="F")
        H = np.empty((r, m), dtype=np.float32, order="F")
        _native.check(self._lib.gpunmf_batch_get(self._h, int(k), W.ctypes.data_as(_P), H.ctypes.data_as(_P)))
        return W, H

    def residuals(self):
        out = np.empty(self.count, dtype=np.float64)
        _native.check(self._lib.gpunmf_batch_residuals(self._h, out.ctypes.data_as(_P)))
        return out

    def set_config(self, k, cfg):
        _native.check(self._lib.gpunmf_batch_set_config(self._h, int(k), int(cfg)))
        self.cfg[k] = cfg

    def commit(self):
        _native.check(self._lib.gpunmf_batch_commit(self._h))

    def reset_factors(self):
        Vs, Ws, Hs = self._keep
        pw = (ctypes.c_void_p * self.count)(*[a.ctypes.data for a in Ws])
        ph = (ctypes.c_void_p * self.count)(*[a.ctypes.data for a in Hs])
        _native.check(self._lib.gpunmf_batch_reset_factors(self._h, pw, ph))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gpunmf_batch_destroy(self._h)
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


def autotune(batch, instances, sample=304, iters=3, seed=0):
    """Pick a tile configuration per (rank class, size class) bucket.

    For each bucket, up to `sample` of its instances form a trial batch that
    is timed (device time, CUDA events) for `iters` iterations under every
    configuration of the bucket's rank class; the fastest is assigned to all
    of the bucket's instances in `batch`.  Returns {bucket: (cfg, {cfg: ms})}.
    """
    ranks = configs()
    rng = np.random.Generator(np.random.PCG64(seed))
    buckets = {}
    for k, (n, m, r) in enumerate(batch.shapes):
        buckets.setdefault((rank_class(r), size_class(n, m)), []).append(k)
    table = {}
    for key, members in sorted(buckets.items()):
        cands = [c for c, rc in enumerate(ranks) if rc == key[0]]
        pick = members if len(members) <= sample else list(rng.choice(members, size=sample, replace=False))
        with Batch([instances[k] for k in pick]) as trial:
            timings = {}
            for c in cands:
                for j in range(trial.count):
                    trial.set_config(j, c)
                trial.commit()
                trial.reset_factors()
                trial.time(iters)  # warm (captures the graph)
                timings[c] = trial.time(iters)
        best = min(timings, key=timings.get)
        table[key] = (best, timings)
        for k in members:
            batch.set_config(k, best)
    batch.commit()
    return table


def run_one_per_instance(instances, iters, eps=1e-8):
    """The comparison path: every instance through the plain FP32 job API, one after another."""
    from .nmf import NMF_MultiplicativeEuclidianDistance
    t0 = time.perf_counter()
    out = []
    for d in instances:
        with NMF_MultiplicativeEuclidianDistance(d["V"], d["W"], d["H"], eps=eps, quality_interval=0) as j:
            j.Iterate(iters)
            out.append((j.GetW(), j.GetH()))
    return out, time.perf_counter() - t0
