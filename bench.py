"""Benchmark: NMF iterations/s on one GB300 (or N independent replicas).

Workload (the headline): multiplicative-update Euclidean NMF, V 8192 x 8192
FP32 = A B + |N(0, 0.01)| with A 8192x64, B 64x8192 ~ Gamma(2, 0.5) (seed 2),
r = 64, W/H U[0,1)+1e-4 (seed 3), eps 1e-9.  A step is one NMF iteration
(H update then W update).  V is 268 MB in FP32 (134 MB as BF16), larger than
the 129 MB L2, so consecutive steps stream it from HBM; no flush is added.

Arms:
  ours (default)     the engine through its C ABI; `value` is device-timed
                     (CUDA events on the job's stream, inputs resident);
                     `e2e` is the same job through the public API from pinned
                     host buffers: create (H2D of V, W, H), K iterations with
                     the per-iteration quality read-back of the reference's
                     DoIteration, then GetW/GetH (D2H), all inside the timed
                     region; `e2e_quality_when_ready` the same job with the
                     quality sampled under the reference's own rule (only
                     when the previous read-back is complete).
  --impl reference   the reference's CPU NMF (HostNMF.h:64-114) on the host
                     cores: the oracle's float transcription, which gives the
                     reference HostNMF's bits (pinned by golden vectors made
                     with the reference's own build), split over all host
                     threads by output element.  Each step is one full-size
                     iteration of the same workload (no slicing, nothing
                     extrapolated).

Multi-GPU: the path does not shard (one factorisation per GPU), so --gpus N
runs N independent replicas (one per rank, launched by torchrun) and reports
the summed iterations/s over the max-over-ranks time.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
FALLBACK_BF16_TFLOPS = 1900.0

METRIC = "NMF iters/s, Euclidean multiplicative update, V 8192x8192, r=64"


def euclid_metric(n, m, r):
    """The headline metric's name for the shape actually run (the default shape gives METRIC)."""
    return "NMF iters/s, Euclidean multiplicative update, V %dx%d, r=%d" % (n, m, r)
GENERATOR = (" (project generator, gpumlib_gb300/inputs.py: splitmix64 counters per element; Marsaglia-Tsang "
             "gamma, Box-Muller normal, inversion / PTRS Poisson)")

# DRAM bytes (read + write) per launch of the dominant kernel, from the committed ncu
# captures of this workload (one --set full capture per precision, see the profiles
# directory): tc_gemm_sk_kernel<64> with the update fused, mean of an H-step and a W-step launch,
# 138.76 MB + 3.75 MB; gemm_f32_kernel (W'V, 19 split-K slices) 275.49 MB + 25.29 MB.
NCU_TRAFFIC_PER_LAUNCH = {"bf16": 142.51e6, "fp32": 300.78e6}
# The same for the KL workload's fused product (tc_kl_gemm_kernel<8>, mean of an H-step and a
# W-step launch: 139.87 MB + 3.94 MB).
KL_NCU_TRAFFIC_PER_LAUNCH = {"bf16": 143.81e6}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--precision", choices=["bf16", "fp32"], default=None)
    p.add_argument("--n", type=int, default=8192)
    p.add_argument("--m", type=int, default=8192)
    p.add_argument("--r", type=int, default=64)
    p.add_argument("--full-job-iters", type=int, default=500,
                   help="iterations of the residual comparison job (0 = skip)")
    p.add_argument("--err-iters", type=int, default=3,
                   help="iterations after which W, H, W H are compared with the FP64 oracle (0 = skip)")
    p.add_argument("--kl-lam-scale", type=float, default=1.0,
                   help="KL workload: Poisson means scaled by this (0.01 gives ~89%% zeros)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--workload", choices=["large_euclidean", "batched", "serving", "kl_counts", "plain_small"],
                   default="large_euclidean")
    p.add_argument("--serve-rate", type=float, default=2000.0)
    p.add_argument("--serve-duration", type=float, default=5.0,
                   help="seconds of arrivals replayed (the full stream is 60)")
    p.add_argument("--serve-drain", type=float, default=240.0,
                   help="seconds each arm may take to finish its admitted and queued jobs after the last arrival")
    p.add_argument("--serve-slots", type=int, default=64)
    p.add_argument("--batch-count", type=int, default=4096)
    p.add_argument("--batch-iters", type=int, default=100)
    p.add_argument("--baseline-sample", type=int, default=128,
                   help="instances run one job at a time through the plain FP32 API for the comparison")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier and max-over-ranks for replicas (gloo on the host; no data-path collective)."""

    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


FP32_SMS = 152


def peak_sm_mhz():
    """The GPU's maximum SM clock (MEASURED_PEAKS.json), else GB300's 2070 MHz."""
    try:
        with open(MEASURED_PEAKS) as f:
            return float(json.load(f)["sm_max_mhz"])
    except Exception:
        return 2070.0


def peaks():
    try:
        with open(MEASURED_PEAKS) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), float(p["bf16_tflops"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, FALLBACK_BF16_TFLOPS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.error = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception as e:  # no nvidia-smi
            self.error = str(e)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def wait_started(self, timeout=10.0):
        """Block until nvidia-smi printed its first sample, so later samples fall in what follows."""
        t0 = time.perf_counter()
        while self.proc and not self.lines and time.perf_counter() - t0 < timeout:
            time.sleep(0.01)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        if self.error or not self.lines:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0,
                    "note": self.error or "no samples"}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# reference arm / CPU baseline
# ---------------------------------------------------------------------------

def timed_repeats(measure, dist, clk, min_seconds=1.0, max_reps=500):
    """Repeat a K-step measurement (measure() returns the device time of exactly K steps, taken with
    CUDA events and synchronised on both sides) so that the timed loops span at least min_seconds and
    the clock sampler, started before them, sees them.  Each repetition is the max over ranks; the
    repetition count comes from the first one (the same on every rank).  Returns the median ms and
    the spread."""
    clk.wait_started()
    first = dist.max(measure())
    reps = int(min(max_reps, max(1, math.ceil(min_seconds * 1e3 / max(first, 1e-3)))))
    times = [first] + [dist.max(measure()) for _ in range(reps - 1)]
    return statistics.median(times), {"repeats": reps, "ms_median": round(statistics.median(times), 4),
                                      "ms_min": round(min(times), 4), "ms_max": round(max(times), 4)}


def workload_config(n, m, r, eps, world, rule="euclidean", **extra):
    """The `config` object of a workload, the same dict on both arms (the engine's arithmetic is
    reported in `dtype` / `precision`, outside it)."""
    cfg = {"workload": "large_euclidean_%dx%d_r%d" % (n, m, r) if rule == "euclidean" else
           "kl_counts_%dx%d_r%d" % (n, m, r), "n": n, "m": m, "r": r, "rule": rule, "eps": eps,
           "parallelism": "replicas" if world > 1 else "single",
           "l2": "inputs larger than L2 (V %d MB fp32 / %d MB bf16 > 129 MB); no flush" %
                 (n * m * 4 >> 20, n * m * 2 >> 20)}
    cfg.update(extra)
    return cfg


def cpu_reference_steps(V, W, H, eps, steps, warmup, min_seconds=0.0, rule=0):
    """Time full-size iterations of the reference's CPU NMF (HostNMF.h:64-150) on all host threads:
    at least `steps` iterations and, if given, at least min_seconds of CPU work.  The oracle's float
    transcription is used: it gives the reference build's bits (golden vectors) and splits each
    product over threads by output element (the reference's HostNMF is single-threaded).
    Returns (iters/s, seconds per iteration, info)."""
    import oracle
    threads = os.cpu_count() or 1
    Wc, Hc = W.copy(order="F"), H.copy(order="F")

    def one():
        nonlocal Wc, Hc
        Wc, Hc = oracle.hostnmf_run(rule, V, Wc, Hc, 1, eps=np.float32(eps), nthreads=threads,
                                    clamp_sums=(rule == 1))

    for _ in range(warmup):
        one()
    t0 = time.perf_counter()
    done = 0
    while done < steps or time.perf_counter() - t0 < min_seconds:
        one()
        done += 1
    dt = time.perf_counter() - t0
    n, m = V.shape
    info = {"kind": "port", "cores": threads,
            "sample": "%d full %dx%d iterations (r=%d) of the same workload, after %d warm-up; the "
                      "reference HostNMF's arithmetic (bit-identical transcription) split over %d host threads"
                      % (done, n, m, W.shape[1], warmup, threads),
            "seconds": round(dt, 3), "iterations": done}
    return done / dt, dt / done, info


def error_vs_f64(rule, V, W, H, eps, iters, gpu_factors):
    """W, H and W H of each precision after `iters` iterations from the workload's W/H, against the
    FP64 oracle's (the GPU classes' rules in double precision) after the same iterations."""
    import oracle
    t0 = time.perf_counter()
    Wd, Hd = oracle.f64_run_blas(rule, V, W, H, iters, eps=eps)
    out = {"iters": iters}
    for prec, (Wg, Hg) in gpu_factors.items():
        out[prec] = {k: float("%.4g" % v) for k, v in oracle.factor_errors(Wg, Hg, Wd, Hd).items()}
    out["oracle"] = "FP64 CPU restatement of the GPU rules (BLAS products), %.1f s" % (time.perf_counter() - t0)
    return out


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def make_workload(n, m, r):
    from gpumlib_gb300 import inputs
    cfg = inputs.large_euclidean(n, m, r)
    return cfg["V"], cfg["W"], cfg["H"], cfg["eps"]


def run_ours(args, rank, world, local, dist):
    import gpumlib_gb300 as g
    from gpumlib_gb300 import _native

    lib = _native.load()
    if g.device_count() < 1:
        raise RuntimeError("no CUDA device")
    precision = args.precision or "bf16"
    n, m, r = args.n, args.m, args.r
    V, W, H, eps = make_workload(n, m, r)
    try:
        nmf = g.NMF_MultiplicativeEuclidianDistance(V, W, H, eps=eps, precision=precision, quality_interval=0)
    except g.GpuNmfError as e:
        if precision == "bf16" and e.status == 4:
            precision = "fp32"
            nmf = g.NMF_MultiplicativeEuclidianDistance(V, W, H, eps=eps, precision=precision, quality_interval=0)
        else:
            raise
    # warm-up, then the timed steps
    nmf.Iterate(args.warmup)
    nmf.Synchronize()
    dist.barrier()
    with ClockSampler(local) as clk:
        t = {}

        def measure():
            t.update(nmf.TimeIterations(args.steps))
            return t["total_ms"]

        ms, rep_info = timed_repeats(measure, dist, clk)
    value = world * args.steps / (ms / 1e3)
    # per-kernel CUDA events around the V-streaming products, in an adjacent loop of the same
    # length on the job's stream (events between kernels would serialise the timed loop above)
    tk = nmf.TimeIterations(args.steps, kernel_timing=True)
    t["kernel_ms"], t["kernel_launches"] = tk["kernel_ms"], tk["kernel_launches"]
    nmf.close()

    # roofline of the dominant kernel (the V-streaming product)
    hbm, _, src = peaks()
    vbytes = 2 if precision == "bf16" else 4
    if precision == "bf16":
        # one half-step kernel: V (BF16) once, the other factor's BF16 copy once, and the updated
        # factor read (FP32), written (FP32) and written again as BF16
        per_launch_bytes = n * m * 2 + n * r * 2 + m * r * (4 + 4 + 2)
    else:
        # the W'V product: V, W and the FP32 partial products of H's shape
        per_launch_bytes = n * m * 4 + (n * r + r * m) * 4 + r * m * 4
    kl = max(1, t["kernel_launches"])
    isolated_ms = t["kernel_ms"] / kl
    if t["launches"] == tk["kernel_launches"]:
        # every launch of the timed region is this kernel (the BF16 path: one launch per half-step),
        # so its average duration is the region's device time over its launches, taken with the
        # programmatic dependent launches overlapping as they do in the job
        avg_ms = ms / t["launches"]
        avg_src = "timed region / launches (all launches are this kernel)"
    else:
        avg_ms = isolated_ms
        avg_src = "CUDA events around each launch in an adjacent loop of the same length"
    achieved = per_launch_bytes / (avg_ms / 1e3) / 1e9
    traffic = NCU_TRAFFIC_PER_LAUNCH.get(precision)
    if precision == "bf16":
        roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(achieved / hbm, 4), "peak_source": src,
                    "kernel": "half-step kernel: V-streaming product with the update fused (tc_gemm_sk_kernel)"}
    else:
        # the FP32 product is bound by the CUDA cores' FMA rate (8.6 GFLOP against 268 MB of V: 32
        # flop per byte), so its roofline is the FP32 peak, computed (no measured figure exists)
        mhz = peak_sm_mhz()
        fp32_peak = FP32_SMS * 128 * 2 * mhz * 1e6 / 1e12
        tfs = 2.0 * n * m * r / (avg_ms / 1e3) / 1e12
        roofline = {"bound": "fp32-simt", "achieved": round(tfs, 2), "peak": round(fp32_peak, 1), "unit": "TFLOP/s",
                    "frac": round(tfs / fp32_peak, 4),
                    "peak_source": "computed: %d SMs x 128 FP32 lanes x 2 flop x %.0f MHz" % (FP32_SMS, mhz),
                    "kernel": "V-streaming product W'V (gemm_f32_kernel)",
                    "hbm_achieved_gbs": round(achieved, 1), "hbm_frac": round(achieved / hbm, 4)}
    roofline.update({"traffic": traffic, "avg_launch_ms": round(avg_ms, 5), "avg_launch_source": avg_src,
                     "isolated_launch_ms": round(isolated_ms, 5), "algorithmic_bytes_per_launch": per_launch_bytes})

    out = {"metric": euclid_metric(n, m, r), "value": round(value, 2), "unit": "iters/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 5), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "bf16" if precision == "bf16" else "f32",
           "precision": precision,
           "data": "synthetic: V = A B + |N(0,0.01)|, A,B ~ Gamma(2,0.5) (seed 2); W,H U[0,1)+1e-4 (seed 3)"
                   "%s" % GENERATOR,
           "config": workload_config(n, m, r, eps, world),
           "clocks": clk.summary(), "timing": rep_info, "gpu_launches": t["launches"], "roofline": roofline}

    # end to end through the public API from pinned host buffers: the workload's own job (the
    # configuration's 500 iterations, --full-job-iters), and a job of --steps iterations beside it
    if not args.no_e2e:
        job_iters = args.full_job_iters or args.steps
        out["e2e"] = run_e2e(lib, g, V, W, H, eps, precision, args, dist, world, iters=job_iters)
        if job_iters != args.steps:
            out["e2e_short_job"] = run_e2e(lib, g, V, W, H, eps, precision, args, dist, world)
        # the same job with QUALITY_WHEN_READY, the sampling rule of the reference's own classes
        out["e2e_quality_when_ready"] = run_e2e(lib, g, V, W, H, eps, precision, args, dist, world,
                                                iters=job_iters, quality_interval=g.QUALITY_WHEN_READY)

    # equal-residual check: a full job in each precision, and the error of W, H and W H against the
    # FP64 oracle after a few iterations from the same start
    if rank == 0:
        precs = ["bf16", "fp32"] if precision == "bf16" else ["fp32"]
        if args.full_job_iters:
            res = {}
            for prec in precs:
                with g.NMF_MultiplicativeEuclidianDistance(V, W, H, eps=eps, precision=prec, quality_interval=0) as j:
                    tt = j.TimeIterations(args.full_job_iters)
                    res[prec] = {"residual": j.Residual(),
                                 "iters_per_s": round(args.full_job_iters / (tt["total_ms"] / 1e3), 2)}
            out["full_job"] = {"iters": args.full_job_iters, **res}
            if "bf16" in res:
                out["full_job"]["residual_gap"] = abs(res["bf16"]["residual"] - res["fp32"]["residual"])
                out["full_job"]["speedup_vs_fp32"] = round(res["bf16"]["iters_per_s"] / res["fp32"]["iters_per_s"], 3)
        if args.err_iters:
            facs = {}
            for prec in precs:
                with g.NMF_MultiplicativeEuclidianDistance(V, W, H, eps=eps, precision=prec, quality_interval=0) as j:
                    j.Iterate(args.err_iters)
                    facs[prec] = (j.GetW(), j.GetH())
            out["err_vs_f64"] = error_vs_f64(0, V, W, H, eps, args.err_iters, facs)

    if rank == 0 and not args.no_cpu_baseline:
        # a bounded sample of about 10 s of host-core work: full-size iterations
        ips, _, info = cpu_reference_steps(V, W, H, eps, steps=1, warmup=1, min_seconds=10.0)
        out["cpu_baseline"] = {"value": ips, "unit": "iters/s", **info}
    return out


def run_e2e(lib, g, V, W, H, eps, precision, args, dist, world, iters=None, make=None, quality_interval=1):
    import ctypes
    n, m = V.shape
    r = W.shape[1]
    bufs = []
    try:
        def pinned(a):
            p = lib.gpunmf_host_alloc(a.nbytes)
            if not p:
                raise MemoryError("pinned allocation failed")
            bufs.append(p)
            arr = np.ctypeslib.as_array((ctypes.c_float * a.size).from_address(p)).reshape(a.shape, order="F")
            arr[...] = a
            return arr
        hV, hW, hH = pinned(V), pinned(W), pinned(H)
        oW = pinned(np.zeros_like(W))
        oH = pinned(np.zeros_like(H))
        from gpumlib_gb300 import _native

        steps = iters or args.steps
        ctor = make or g.NMF_MultiplicativeEuclidianDistance

        def job(iters):
            nmf = ctor(hV, hW, hH, eps=eps, precision=precision, quality_interval=quality_interval)
            for _ in range(iters):
                nmf.DoIteration()            # quality read-back (4 bytes D2H) per sampled iteration
                nmf.QualityImprovement()
            _native.check(lib.gpunmf_get_w(nmf._h, oW.ctypes.data_as(ctypes.c_void_p)))
            _native.check(lib.gpunmf_get_h(nmf._h, oH.ctypes.data_as(ctypes.c_void_p)))
            return nmf

        # one untimed job of `warmup` iterations first: the kernels this path alone uses (quality,
        # conversions) are loaded on their first launch, which is not part of a job's cost
        job(max(1, args.warmup)).close()
        dist.barrier()
        t0 = time.perf_counter()
        nmf = job(steps)
        dt = time.perf_counter() - t0
        nmf.close()
        dt = dist.max(dt)
        h2d = V.nbytes + W.nbytes + H.nbytes
        d2h = W.nbytes + H.nbytes + 4 * steps
        sampling = ("the quality sampled every iteration (the default: deterministic)" if quality_interval == 1 else
                    "the quality sampled under the reference's rule (an iteration samples when the previous "
                    "read-back is complete; d2h counts every iteration's 4 bytes, an upper bound)")
        return {"value": round(world * steps / dt, 2), "unit": "iters/s",
                "h2d_bytes_per_step": h2d // steps, "d2h_bytes_per_step": d2h // steps,
                "note": "one job of %d iterations from pinned host buffers, after one untimed warm-up job: create "
                        "(V, W, H read from the host), DoIteration() + QualityImprovement() per iteration with %s, "
                        "GetW/GetH (D2H); bytes amortised per step" % (steps, sampling)}
    finally:
        for p in bufs:
            lib.gpunmf_host_free(p)


# ---------------------------------------------------------------------------
# plain FP32 workload: V 1024 x 512, r = 16, 200 iterations, residual every iteration
# ---------------------------------------------------------------------------
PLAIN_METRIC = "NMF iters/s, plain FP32 Euclidean multiplicative update, V 1024x512, r=16, 200 iterations"


def run_plain(args, rank, world, local, dist):
    import gpumlib_gb300 as g
    from gpumlib_gb300 import _native, inputs
    import oracle

    lib = _native.load()
    cfg = inputs.plain_euclidean_1024x512()
    V, W, H, eps, iters = cfg["V"], cfg["W"], cfg["H"], cfg["eps"], cfg["iters"]
    n, m = V.shape
    r = cfg["r"]
    prec = args.precision or "fp32"
    # device-timed: a step is one iteration (inputs resident), the timed loop repeated as for the
    # large workload
    nmf = g.NMF_MultiplicativeEuclidianDistance(V, W, H, eps=eps, precision=prec, quality_interval=0)
    nmf.Iterate(args.warmup)
    nmf.Synchronize()
    dist.barrier()
    with ClockSampler(local) as clk:
        t = {}

        def measure():
            t.update(nmf.TimeIterations(args.steps))
            return t["total_ms"]

        ms, rep_info = timed_repeats(measure, dist, clk)
    nmf.close()
    value = world * args.steps / (ms / 1e3)
    out = {"metric": PLAIN_METRIC, "value": round(value, 2), "unit": "iters/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 5),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "bf16" if prec == "bf16" else "f32", "precision": prec,
           "data": "synthetic: V U[0,1) (seed 0); W,H U[0,1)+1e-4 (seed 1)",
           "config": {"workload": "plain_euclidean_1024x512_r16", "n": n, "m": m, "r": r, "rule": "euclidean",
                      "eps": eps, "iters": iters, "parallelism": "replicas" if world > 1 else "single",
                      "l2": "V 2 MB fits L2: a launch-bound workload; no flush"},
           "clocks": clk.summary(), "timing": rep_info, "gpu_launches": t["launches"]}
    if rank == 0:
        # the whole 200-iteration job with the residual read after every iteration, against the
        # reference HostNMF's trajectory (its own build where present, else the bit-identical port)
        traj = []
        with g.NMF_MultiplicativeEuclidianDistance(V, W, H, eps=eps, precision=prec, quality_interval=0) as j:
            for _ in range(iters):
                j.DoIteration()
                traj.append(j.Residual())
            Wg, Hg = j.GetW(), j.GetH()
        threads = os.cpu_count() or 1
        Wo, Ho, otraj = oracle.hostnmf_run(0, V, W, H, iters, eps=np.float32(eps), nthreads=threads, residuals=True)
        traj = np.array(traj)
        out["residual_per_iteration"] = [float("%.7g" % x) for x in traj]
        out["vs_reference_cpu"] = {
            "max_rel_residual_diff": float(np.max(np.abs(traj - otraj) / otraj)),
            "WH": oracle.factor_errors(Wg, Hg, Wo.astype(np.float64), Ho.astype(np.float64))["WH"],
            "against": "reference HostNMF arithmetic (float transcription, golden-pinned), same eps"}
        if not args.no_cpu_baseline:
            # the reference's CPU NMF timed over the full 200-iteration job (its own build, which has
            # its eps built in at 1e-8 -- the cost does not depend on it -- where present)
            if oracle.ref() is not None:
                t0 = time.perf_counter()
                oracle.reference_run(0, V, W, H, iters)
                dt = time.perf_counter() - t0
                kind, cores = "reference", 1
            else:
                t0 = time.perf_counter()
                oracle.hostnmf_run(0, V, W, H, iters, eps=np.float32(eps), nthreads=threads)
                dt = time.perf_counter() - t0
                kind, cores = "port", threads
            out["cpu_baseline"] = {"value": iters / dt, "unit": "iters/s", "kind": kind, "cores": cores,
                                   "sample": "the full %d-iteration job" % iters, "seconds": round(dt, 3)}
        if not args.no_e2e:
            out["e2e"] = run_e2e(lib, g, V, W, H, eps, prec, args, dist, world, iters=iters)
    return out


# ---------------------------------------------------------------------------
# batched workload: 4096 uneven small Euclidean instances, 100 iterations each
# ---------------------------------------------------------------------------
BATCH_METRIC = "batched NMF jobs/s (4096 uneven Euclidean instances, 100 iterations each)"


def run_batched(args, rank, world, local, dist):
    import gpumlib_gb300 as g
    from gpumlib_gb300 import batch as gb
    from gpumlib_gb300 import inputs

    count, iters = args.batch_count, args.batch_iters
    insts = [inputs.batched_instance(i) for i in range(count)]
    t0 = time.perf_counter()
    b = gb.Batch(insts, eps=1e-8)
    create_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    table = gb.autotune(b, insts)
    tune_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        b.reset_factors()
        b.time(iters)
    dist.barrier()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            b.reset_factors()
            times.append(b.time(iters))
    ms = dist.max(sum(times) / len(times))
    value = world * count / (ms / 1e3)
    res = b.residuals()
    # end to end through the public API: create from host buffers, run, read every W and H back
    e2e = None
    if not args.no_e2e:
        t0 = time.perf_counter()
        with gb.Batch(insts, eps=1e-8) as be:
            for k in range(count):
                be.set_config(k, b.cfg[k])
            be.commit()
            be.run(iters)
            outs = [be.get(k) for k in range(count)]
        e2e_s = dist.max(time.perf_counter() - t0)
        h2d = sum(d["V"].nbytes + d["W"].nbytes + d["H"].nbytes for d in insts)
        d2h = sum(w.nbytes + h.nbytes for w, h in outs)
        e2e = {"value": round(world * count / e2e_s, 1), "unit": "jobs/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h,
               "note": "a step is the whole batch: create from host (H2D), one persistent launch, all W/H read back"}
    b.close()
    # comparison: one job per instance through the plain FP32 job API (a sample, largest and smallest mixed)
    sample = [insts[k] for k in range(0, count, max(1, count // args.baseline_sample))][:args.baseline_sample]
    _, base_s = gb.run_one_per_instance(sample, iters)
    base_jobs_s = len(sample) / base_s
    fp32_mhz = peak_sm_mhz()
    fp32_peak = FP32_SMS * 128 * 2 * fp32_mhz * 1e6 / 1e12
    total_madds = sum(2 * n * m * r + 2 * r * r * (n + m) for (n, m, r) in (d["V"].shape + (d["W"].shape[1],)
                                                                          for d in insts)) * iters
    out = {"metric": BATCH_METRIC, "value": round(value, 1), "unit": "jobs/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic: per instance i (seed 1000+i) m~U{32..512}, n~U{32..1024}, r in {4,8,16,32}, V U[0,1)"
                   "%s" % GENERATOR,
           "config": {"workload": "batched_%d_uneven_iters%d" % (count, iters), "instances": count,
                      "iters": iters, "rule": "euclidean", "precision": "fp32",
                      "l2": "each step re-reads every instance's V 2x per iteration; working set %.2f GB > L2" %
                            (sum(d["V"].nbytes for d in insts) / 1e9)},
           "clocks": clk.summary(), "gpu_launches": args.steps,
           "roofline": {"bound": "fp32-simt", "achieved": round(2 * total_madds / (ms / 1e3) / 1e12, 2),
                        "peak": round(fp32_peak, 1), "unit": "TFLOP/s",
                        "frac": round(2 * total_madds / (ms / 1e3) / 1e12 / fp32_peak, 4),
                        "peak_source": "computed: %d SMs x 128 FP32 lanes x 2 flop x %.0f MHz (no measured FP32 "
                                       "figure exists for this GPU)" % (FP32_SMS, fp32_mhz),
                        "note": "FP32 CUDA-core arithmetic; V served mostly from L2 (instances in flight)"},
           "autotune": {"%d/%d" % k: v[0] for k, v in table.items()}, "autotune_s": round(tune_s, 2),
           "create_s": round(create_s, 2),
           "residual": {"median": float(np.median(res)), "max": float(np.max(res))},
           "one_job_per_instance": {"jobs_per_s": round(base_jobs_s, 2), "sample": len(sample),
                                    "speedup": round(value / base_jobs_s, 1)}}
    if e2e:
        out["e2e"] = e2e
    return out


# ---------------------------------------------------------------------------
# KL workload: V 16384 x 4096 Poisson counts, r = 128
# ---------------------------------------------------------------------------
KL_METRIC = "NMF iters/s, KL multiplicative update, V 16384x4096 Poisson counts, r=128"


def run_kl(args, rank, world, local, dist):
    import gpumlib_gb300 as g
    from gpumlib_gb300 import inputs

    cfg = inputs.kl_counts(lam_scale=args.kl_lam_scale)
    V, W, H, eps = cfg["V"], cfg["W"], cfg["H"], cfg["eps"]
    n, m = V.shape
    r = cfg["r"]
    prec = args.precision or "bf16"
    nmf = g.NMF_MultiplicativeDivergence(V, W, H, eps=eps, precision=prec, quality_interval=0)
    nmf.Iterate(args.warmup)
    nmf.Synchronize()
    dist.barrier()
    with ClockSampler(local) as clk:
        t = {}

        def measure():
            t.update(nmf.TimeIterations(args.steps))
            return t["total_ms"]

        ms, rep_info = timed_repeats(measure, dist, clk)
    value = world * args.steps / (ms / 1e3)
    tk = nmf.TimeIterations(args.steps, kernel_timing=True)
    nmf.close()
    hbm, bf16_tf, src = peaks()
    vbytes = 2 if prec == "bf16" else 4
    per_launch = n * m * vbytes + (n + m) * r * vbytes * 2
    flops = 4.0 * n * m * r  # S = W H block products and the numerator product
    avg_ms = tk["kernel_ms"] / max(1, tk["kernel_launches"])
    gbs = per_launch / (avg_ms / 1e3) / 1e9
    tfs = flops / (avg_ms / 1e3) / 1e12
    if prec == "bf16" and tfs / bf16_tf > gbs / hbm:
        roof = {"bound": "tensor", "achieved": round(tfs, 1), "peak": bf16_tf, "unit": "TFLOP/s",
                "frac": round(tfs / bf16_tf, 4)}
    else:
        roof = {"bound": "hbm", "achieved": round(gbs, 1), "peak": hbm, "unit": "GB/s", "frac": round(gbs / hbm, 4)}
    roof.update({"traffic": KL_NCU_TRAFFIC_PER_LAUNCH.get(prec), "peak_source": src, "avg_launch_ms": round(avg_ms, 5),
                 "kernel": "fused KL product (S = WH -> V/(S+eps) -> numerator)" if prec == "bf16" else
                           "KL ratio SGEMM", "hbm_frac": round(gbs / hbm, 4),
                 "tensor_frac": round(tfs / bf16_tf, 4) if prec == "bf16" else None})
    out = {"metric": KL_METRIC, "value": round(value, 2), "unit": "iters/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 5), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "bf16" if prec == "bf16" else "f32",
           "precision": prec,
           "data": "synthetic: V ~ Poisson(%sP Q), P 16384x128, Q 128x4096 ~ Gamma(0.3,1) (seed 4); W,H U[0,1)+1e-4 "
                   "(seed 5)%s" % ("" if args.kl_lam_scale == 1.0 else "%g " % args.kl_lam_scale, GENERATOR),
           "config": workload_config(n, m, r, eps, world, rule="kl", lam_scale=args.kl_lam_scale,
                                     zero_fraction=round(float(np.mean(V == 0)), 5)),
           "clocks": clk.summary(), "timing": rep_info, "gpu_launches": t["launches"], "roofline": roof}
    if args.kl_lam_scale != 1.0:
        out["config"]["workload"] += "_lam%g" % args.kl_lam_scale
    if rank == 0:
        precs = ["bf16", "fp32"] if prec == "bf16" else ["fp32"]
        if args.full_job_iters:
            iters = min(args.full_job_iters, cfg["iters"])
            res = {}
            for pr in precs:
                with g.NMF_MultiplicativeDivergence(V, W, H, eps=eps, precision=pr, quality_interval=0) as j:
                    tt = j.TimeIterations(iters)
                    res[pr] = {"residual": j.Residual(), "kl_objective": j.ObjectiveKL(),
                               "iters_per_s": round(iters / (tt["total_ms"] / 1e3), 2)}
            out["full_job"] = {"iters": iters, **res}
            if "bf16" in res:
                out["full_job"]["residual_gap"] = abs(res["bf16"]["residual"] - res["fp32"]["residual"])
                out["full_job"]["speedup_vs_fp32"] = round(res["bf16"]["iters_per_s"] / res["fp32"]["iters_per_s"], 2)
        if args.err_iters:
            facs = {}
            for pr in precs:
                with g.NMF_MultiplicativeDivergence(V, W, H, eps=eps, precision=pr, quality_interval=0) as j:
                    j.Iterate(args.err_iters)
                    facs[pr] = (j.GetW(), j.GetH())
            out["err_vs_f64"] = error_vs_f64(1, V, W, H, eps, args.err_iters, facs)
    return out


# ---------------------------------------------------------------------------
# serving workload: Poisson arrivals, continuous batching
# ---------------------------------------------------------------------------
SERVE_METRIC = "NMF serving jobs/s and p50/p99 latency (Poisson arrivals, n,m log-uniform [64,4096], r U{8..64})"


def run_serving(args, rank, world, local, dist):
    from gpumlib_gb300 import inputs, serve

    trace = inputs.serving_trace(rate=args.serve_rate, duration=args.serve_duration, seed=7)
    out_arms = {}
    with ClockSampler(local) as clk:
        for name, prec, slots in (("bf16", "bf16", args.serve_slots), ("fp32", "fp32", args.serve_slots),
                                  ("one_job_at_a_time_fp32", "fp32", 1)):
            tr = trace if slots > 1 else trace[:max(1, len(trace) // 20)]
            with serve.Server(slots=slots, hbm_budget_gb=150.0, precision=prec, check_every=10, tol=1e-3,
                              max_iters=500) as s:
                results, makespan, unfinished = serve.replay(s, tr, drain_timeout_s=args.serve_drain)
                lat = serve.latency_summary(results, unfinished, makespan)
            ok = [r for r in results if r["status"] == 0]
            out_arms[name] = {"jobs": len(tr), "completed": len(ok), "unfinished": len(unfinished),
                              "makespan_s": round(makespan, 3), "jobs_per_s": round(len(ok) / makespan, 2),
                              "latency": lat,
                              "converged_frac": round(sum(r["residual"] <= 1e-3 for r in ok) / max(1, len(ok)), 3),
                              "iters_mean": round(float(np.mean([r["iters"] for r in ok])) if ok else 0.0, 1),
                              "admission_wait_p50_s": float(np.percentile([r["t_admit"] - r["t_submit"] for r in ok], 50))
                              if ok else None}
    main = out_arms["bf16"]
    return {"metric": SERVE_METRIC, "value": main["jobs_per_s"], "unit": "jobs/s", "n_gpus": world,
            "steps": 1, "warmup": 0, "ms_per_step": round(main["makespan_s"] * 1e3, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
            "data": "synthetic: per-job V = A B + |N(0,0.01)|, A,B U[0,1) rank r, generated on the device "
                    "from the job seed",
            "config": {"workload": "serving_poisson_%g_per_s_%gs" % (args.serve_rate, args.serve_duration),
                       "rate": args.serve_rate, "duration_s": args.serve_duration, "kl_fraction": 0.3,
                       "tol": 1e-3, "max_iters": 500, "hbm_budget_gb": 150, "slots": args.serve_slots,
                       "grid_policy": "BF16 jobs: one CTA per 128x128 block, at most 24 CTAs (server default)",
                       "drain_timeout_s": args.serve_drain},
            "clocks": clk.summary(), "arms": out_arms,
            "note": "one_job_at_a_time_fp32 replays the first 5% of the trace through a single slot"}


def reference_gpu_classes(V, W, H, iters, warmup):
    """The reference's own GPU class NMF_MultiplicativeEuclidianDistance (built from its sources for
    sm_103a with cuBLAS) on the same workload: DoIteration() calls per second, its quality sampling
    included, as the class runs it.  Its epsilon is fixed at 1e-8 (nmf_kernels.h:34)."""
    os.environ["NVIDIA_TF32_OVERRIDE"] = "0"   # plain FP32 SGEMM, as the reference's cuBLAS calls ask
    try:
        import oracle
        if oracle.reference_gpu() is None:
            return {"unavailable": "no reference sources (tree or staged copy) to build its GPU classes from"}
        _, _, sec = oracle.reference_gpu_run(0, V, W, H, iters, warmup=warmup)
    except Exception as exc:   # reported, not fatal: the CPU reference is the arm's value
        return {"unavailable": "%s: %s" % (type(exc).__name__, exc)}
    return {"value": round(iters / sec, 3), "unit": "iters/s", "iterations": iters, "warmup": warmup,
            "seconds": round(sec, 4), "precision": "fp32 (cuBLAS SGEMM, TF32 off)", "eps": 1e-8,
            "what": "reference NMF_MultiplicativeEuclidianDistance::DoIteration() on the GPU, built from its "
                    "sources for sm_103a; wall time between device synchronisations"}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    n, m, r = args.n, args.m, args.r
    V, W, H, eps = make_workload(n, m, r)
    # every step (and every warm-up step) is one full-size iteration
    ips, sec, info = cpu_reference_steps(V, W, H, eps, steps=max(1, args.steps), warmup=max(0, args.warmup))
    gpu_classes = reference_gpu_classes(V, W, H, iters=max(20, args.steps), warmup=max(3, args.warmup))
    return {"impl": "reference", "metric": euclid_metric(n, m, r), "value": ips, "unit": "iters/s", "n_gpus": world,
            "steps": info["iterations"], "warmup": args.warmup, "ms_per_step": round(sec * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "precision": "fp32",
            "data": "synthetic (same workload as the engine arm)",
            "config": workload_config(n, m, r, eps, world),
            "cpu_baseline": {"value": ips, "unit": "iters/s", **info},
            "e2e": {"value": ips, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_classes": gpu_classes}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        out = run_reference(args, rank, world)
        if out is not None:
            print(json.dumps(out))
        return 0
    if world > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    dist = Dist(world)
    try:
        if args.workload == "batched":
            out = run_batched(args, rank, world, local, dist)
        elif args.workload == "serving":
            out = run_serving(args, rank, world, local, dist)
        elif args.workload == "kl_counts":
            out = run_kl(args, rank, world, local, dist)
        elif args.workload == "plain_small":
            out = run_plain(args, rank, world, local, dist)
        else:
            out = run_ours(args, rank, world, local, dist)
    finally:
        dist.close()
    if rank == 0:
        print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
