"""ctypes access to the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg and
reference arm may use this package, and only as the checker or as the
reference being timed.  ``orc()`` loads the float/double restatement built
from oracle/nmf_oracle.c; ``ref()`` loads the reference's own HostNMF built
from its sources (present only where the reference tree was available at
build time); ``reference_gpu()`` loads the reference's own GPU classes, built
for sm_103a from its sources or their staged copy.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_orc = None
_ref = None


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def orc():
    global _orc
    if _orc is None:
        path = os.path.join(_build.LIB_DIR, "liborc.so")
        if not os.path.exists(path):
            path = _build.build_oracle()
        lib = ctypes.CDLL(path)
        vp, i, f, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double
        lib.orc_hostnmf_me_iter.argtypes = [i, i, i, vp, vp, vp, i, f, vp, i]
        lib.orc_hostnmf_md_iter.argtypes = [i, i, i, vp, vp, vp, i, f, i, vp, i]
        lib.orc_hostnmf_ae_iter.argtypes = [i, i, i, vp, vp, vp, i, i, vp, i]
        lib.orc_hostnmf_ad_iter.argtypes = [i, i, i, vp, vp, vp, i, f, i, vp, i]
        lib.orc_hostnmf_wh.argtypes = [i, i, i, vp, vp, vp, i]
        lib.orc_f64_me_iter.argtypes = [i, i, i, vp, vp, vp, i, d, vp, i]
        lib.orc_f64_md_iter.argtypes = [i, i, i, vp, vp, vp, i, d, vp, i]
        lib.orc_f64_md_iter.restype = i
        lib.orc_quality.argtypes = [ctypes.c_long, vp, vp, f]
        lib.orc_quality.restype = d
        lib.orc_residual.argtypes = [i, i, i, vp, vp, vp, i]
        lib.orc_residual.restype = d
        _orc = lib
    return _orc


def ref():
    """The reference's HostNMF library, or None when it was not built here."""
    global _ref
    if _ref is None:
        path = os.path.join(_build.REF_DIR, "libhostnmf_ref.so")
        if not os.path.exists(path):
            if not _build.reference_available():
                return None
            path = _build.build_ref()
        lib = ctypes.CDLL(path)
        vp, i = ctypes.c_void_p, ctypes.c_int
        lib.ref_hostnmf_run.argtypes = [i, i, i, i, vp, vp, vp, i, i, vp]
        lib.ref_hostnmf_run.restype = i
        lib.ref_hostnmf_time.argtypes = [i, i, i, i, vp, vp, vp, i]
        lib.ref_hostnmf_time.restype = ctypes.c_double
        _ref = lib
    return _ref


_ref_gpu = None


def reference_gpu():
    """The reference's own GPU NMF classes, built from its sources for sm_103a with cuBLAS
    (oracle/build.py: build_ref_gpu), or None where neither the reference tree nor its staged
    copy is present.  Needs a GPU to run."""
    global _ref_gpu
    if _ref_gpu is None:
        path = _build.build_ref_gpu()
        if path is None:
            return None
        lib = ctypes.CDLL(path)
        vp, i = ctypes.c_void_p, ctypes.c_int
        lib.refgpu_init.argtypes = []
        lib.refgpu_init.restype = i
        lib.refgpu_run.argtypes = [i, i, i, i, vp, vp, vp, i, i, vp]
        lib.refgpu_run.restype = i
        _ref_gpu = lib
    return _ref_gpu


def reference_gpu_run(rule, V, W, H, iters, warmup=0):
    """(W, H, seconds): the reference's NMF_MultiplicativeEuclidianDistance (rule 0) or
    NMF_MultiplicativeDivergence (rule 1) constructed from (V, W, H), `warmup` then `iters`
    DoIteration() calls; seconds is the wall time of the `iters` calls between device
    synchronisations."""
    lib = reference_gpu()
    if lib is None:
        raise RuntimeError("the reference's GPU classes are not available (no reference sources)")
    V = _f32_in(V); W = _f32(W); H = _f32(H)
    n, m = V.shape
    r = W.shape[1]
    sec = ctypes.c_double(0.0)
    rc = lib.refgpu_run(rule, n, m, r, _p(V), _p(W), _p(H), warmup, iters, ctypes.byref(sec))
    if rc != 0:
        raise RuntimeError("reference GPU NMF failed with code %d" % rc)
    return W, H, sec.value


def _f32(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float32)).copy(order="F")


def _f32_in(a):
    """A read-only operand (V): used as is when already float32 column-major, else converted."""
    a = np.asarray(a)
    if a.dtype == np.float32 and a.flags.f_contiguous:
        return a
    return np.asfortranarray(a, dtype=np.float32)


def hostnmf_run(rule, V, W, H, iters, updateW=True, eps=1e-8, clamp_sums=False, nthreads=1,
                residuals=False, skip_h=False):
    """Float transcription of HostNMF; rule 0 multiplicative Euclidean, 1 multiplicative KL,
    2 additive Euclidean (skip_h: the GPU class's H step that leaves H unchanged), 3 additive KL.
    Returns (W, H[, resid])."""
    lib = orc()
    V = _f32_in(V); W = _f32(W); H = _f32(H)
    n, m = V.shape
    r = W.shape[1]
    if rule in (0, 2):
        ws = np.empty(2 * r * m + r * r + 2 * n * r, dtype=np.float32)
    else:
        ws = np.empty(n * m, dtype=np.float32)
    res = []
    for _ in range(iters):
        if rule == 0:
            lib.orc_hostnmf_me_iter(n, m, r, _p(V), _p(W), _p(H), int(updateW), eps, _p(ws), nthreads)
        elif rule == 1:
            lib.orc_hostnmf_md_iter(n, m, r, _p(V), _p(W), _p(H), int(updateW), eps, int(clamp_sums),
                                    _p(ws), nthreads)
        elif rule == 2:
            lib.orc_hostnmf_ae_iter(n, m, r, _p(V), _p(W), _p(H), int(updateW), int(skip_h), _p(ws), nthreads)
        else:
            lib.orc_hostnmf_ad_iter(n, m, r, _p(V), _p(W), _p(H), int(updateW), eps, int(clamp_sums),
                                    _p(ws), nthreads)
        if residuals:
            res.append(residual(V, W, H, nthreads))
    return (W, H, np.array(res)) if residuals else (W, H)


def f64_run(rule, V, W, H, iters, updateW=True, eps=1e-8, nthreads=1):
    """Double-precision GPU-semantics rules; returns float64 (W, H)."""
    lib = orc()
    V = np.asfortranarray(np.asarray(V, dtype=np.float64))
    W = np.asfortranarray(np.asarray(W, dtype=np.float64)).copy(order="F")
    H = np.asfortranarray(np.asarray(H, dtype=np.float64)).copy(order="F")
    n, m = V.shape
    r = W.shape[1]
    if rule == 0:
        ws = np.empty(2 * r * m + r * r + 2 * n * r, dtype=np.float64)
    else:
        ws = np.empty(n * m + r, dtype=np.float64)
    for _ in range(iters):
        if rule == 0:
            lib.orc_f64_me_iter(n, m, r, _p(V), _p(W), _p(H), int(updateW), eps, _p(ws), nthreads)
        else:
            if lib.orc_f64_md_iter(n, m, r, _p(V), _p(W), _p(H), int(updateW), eps, _p(ws), nthreads) != 0:
                raise ValueError("r too large for the oracle")
    return W, H


def f64_run_blas(rule, V, W, H, iters, updateW=True, eps=1e-8):
    """The same FP64 rules as f64_run with the products formed by numpy's BLAS (any summation order;
    in FP64 that moves results by ~1e-13, far below what they check).  Used where f64_run's loops
    would take minutes: full-size accuracy checks.
      Euclidean (nmf_multiplicative_euclidian.cpp:29-67, nmf_kernels.cu:43-47):
        H *= W'V / (W'W H + eps);  W *= V H' / (W H H' + eps)
      KL (nmf_multiplicative_divergence.cpp:29-50, nmf_kernels.cu:63-233,247-341):
        H *= W'(V / (W H + eps)) / max(colsum W, eps);  W *= (V / (W H + eps)) H' / max(rowsum H, eps)
    Returns float64 (W, H)."""
    V = np.asarray(V, dtype=np.float64)
    W = np.array(W, dtype=np.float64)
    H = np.array(H, dtype=np.float64)
    for _ in range(iters):
        if rule == 0:
            H *= (W.T @ V) / ((W.T @ W) @ H + eps)
            if updateW:
                W *= (V @ H.T) / (W @ (H @ H.T) + eps)
        elif rule == 1:
            R = V / (W @ H + eps)
            H *= (W.T @ R) / np.maximum(W.sum(axis=0), eps)[:, None]
            if updateW:
                R = V / (W @ H + eps)
                W *= (R @ H.T) / np.maximum(H.sum(axis=1), eps)[None, :]
            del R
        else:
            raise ValueError("rule %d has no FP64 restatement" % rule)
    return W, H


def factor_errors(Wg, Hg, Wd, Hd):
    """Relative Frobenius errors of W, H and W H against a reference (W H formed in FP64)."""
    def rel(a, b):
        a = np.asarray(a, dtype=np.float64)
        b = np.asarray(b, dtype=np.float64)
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
    Wg = np.asarray(Wg, dtype=np.float64)
    Hg = np.asarray(Hg, dtype=np.float64)
    return {"W": rel(Wg, Wd), "H": rel(Hg, Hd), "WH": rel(Wg @ Hg, Wd @ Hd)}


def hostnmf_wh(W, H, nthreads=1):
    W = _f32(W); H = _f32(H)
    n, r = W.shape
    m = H.shape[1]
    WH = np.empty((n, m), dtype=np.float32, order="F")
    orc().orc_hostnmf_wh(n, m, r, _p(W), _p(H), _p(WH), nthreads)
    return WH


def quality(V, WH, eps=1e-8):
    V = _f32(V); WH = _f32(WH)
    return orc().orc_quality(V.size, _p(V), _p(WH), eps)


def residual(V, W, H, nthreads=1):
    V = _f32(V); W = _f32(W); H = _f32(H)
    n, m = V.shape
    return orc().orc_residual(n, m, W.shape[1], _p(V), _p(W), _p(H), nthreads)


def reference_run(rule, V, W, H, iters, updateW=True, residuals=False):
    """Run the reference's own HostNMF (built from its sources); None if unavailable."""
    lib = ref()
    if lib is None:
        return None
    V = _f32(V); W = _f32(W); H = _f32(H)
    n, m = V.shape
    r = W.shape[1]
    res = np.zeros(iters, dtype=np.float64)
    rc = lib.ref_hostnmf_run(rule, n, m, r, _p(V), _p(W), _p(H), iters, int(updateW),
                             _p(res) if residuals else None)
    if rc != 0:
        raise RuntimeError("ref_hostnmf_run failed")
    return (W, H, res) if residuals else (W, H)


class QualityLag:
    """NMF::DetermineQualityImprovement (nmf_base.h:70-89) with every read-back complete: the value
    read at an iteration is the quality sampled at the previous one (0.0 before the first sample),
    and the improvement is set from the third sample on.  All values are float32 as in the reference."""

    def __init__(self):
        self.times = 0
        self.last = np.float32(-1.0)
        self.delta = np.float32(1.0)
        self.value = np.float32(0.0)

    def sample(self, new_value):
        q = self.value
        if self.times > 2:
            self.delta = np.float32(q - self.last)
        self.times += 1
        if self.times <= 3:
            self.times += 1
        self.last = q
        self.value = np.float32(new_value)


def grouped_run(rule, V, W, H, group, tol, max_iters, eps=1e-8, nthreads=1, iters_per_block=None):
    """TrainUsingGroups (src/examples/FacesNMF/FacesNMFDlg.cpp:582-656) over the float oracle.

    V's first floor(m/group)*group columns are split into blocks of `group` columns; block s has rank
    rs = floor(r / blocks) and starts from W[:, s*rs:(s+1)*rs] and the diagonal block
    H[s*rs:(s+1)*rs, s*group:(s+1)*group] (the reference draws fresh random factors instead).  Each
    block iterates until its QualityImprovement() changes to a value below tol (the reference's loop,
    :605-629) or max_iters.  Its W fills the block's columns of W; its H fills the block's rows of
    the block's columns of H, zeros elsewhere in those columns (:632-651).  Rule 4 is the additive
    Euclidean rule with the H step skipped.  iters_per_block runs exactly those counts instead of the
    test.  Returns (W, H, iterations per block, deltas per block).
    """
    V = _f32(V)
    W = _f32(W).copy(order="F")
    H = _f32(H).copy(order="F")
    n, m = V.shape
    r = W.shape[1]
    blocks = m // group
    rs = r // blocks
    iters_out, deltas_out = [], []
    for s in range(blocks):
        Vs = np.asfortranarray(V[:, s * group:(s + 1) * group])
        Ws = np.asfortranarray(W[:, s * rs:(s + 1) * rs])
        Hs = np.asfortranarray(H[s * rs:(s + 1) * rs, s * group:(s + 1) * group])
        lag = QualityLag()
        prev = lag.delta
        deltas = []
        k = 0
        limit = max_iters if iters_per_block is None else iters_per_block[s]
        while k < limit:
            lag.sample(quality(Vs, hostnmf_wh(Ws, Hs), eps))
            Ws, Hs = hostnmf_run(2 if rule == 4 else rule, Vs, Ws, Hs, 1, eps=eps, clamp_sums=True,
                                 nthreads=nthreads, skip_h=(rule == 4))
            k += 1
            q = lag.delta
            deltas.append(float(q))
            if q != prev and iters_per_block is None:
                if q < tol:
                    break
                prev = q
        W[:, s * rs:(s + 1) * rs] = Ws
        H[:, s * group:(s + 1) * group] = 0.0
        H[s * rs:(s + 1) * rs, s * group:(s + 1) * group] = Hs
        iters_out.append(k)
        deltas_out.append(deltas)
    return W, H, iters_out, deltas_out
