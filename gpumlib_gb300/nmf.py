"""Python mirror of GPUMLib's NMF classes over the C ABI.

Same class names, constructor forms and methods as
src/algorithms/nmf/nmf_base.h:45-151,
src/algorithms/nmf/nmf_multiplicative_euclidian.h:51-65,
src/algorithms/nmf/nmf_multiplicative_divergence.h:48-58,
src/algorithms/nmf/nmf_additive_euclidian.h:35-67 and
src/algorithms/nmf/nmf_additive_divergence.h:35-60:

    nmf = NMF_MultiplicativeEuclidianDistance(V, r)        # random W, H
    nmf = NMF_MultiplicativeEuclidianDistance(V, W, H)     # given W, H
    nmf.DoIteration(updateW=True)
    nmf.GetW(); nmf.GetH(); nmf.GetWH(); nmf.QualityImprovement()

Matrices are 2-D numpy float32 arrays (rows x columns); they are handed to
the library column-major, as the reference requires (nmf_base.h:92,109).
Additions beyond the reference: ``Iterate(k)``, ``Residual()`` (FP64
relative Frobenius residual on the GPU), ``ObjectiveKL()``, an ``eps``
argument (the reference hard-codes 1e-8) and a ``precision`` argument
("fp32" = the drop-in path, "bf16" = tensor-core products).
"""
import ctypes

import numpy as np

from . import _native

EUCLIDEAN = 0
DIVERGENCE = 1
ADDITIVE_EUCLIDEAN = 2
ADDITIVE_DIVERGENCE = 3
ADDITIVE_EUCLIDEAN_FIXED_H = 4
PRECISIONS = {"fp32": 0, "bf16": 1}
REFERENCE_EPS = np.float32(1e-8)
# quality_interval / SetQualityInterval: sample only when the previous sample's read-back is complete,
# never waiting (the reference's rule, nmf_base.h:71); k > 0 samples every k-th iteration, 0 never
QUALITY_WHEN_READY = -1


def _fortran32(a):
    a = np.asarray(a, dtype=np.float32)
    if a.ndim != 2:
        raise ValueError("matrices must be 2-D")
    return np.asfortranarray(a)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class NMF:
    """Base class (nmf_base.h:45).  Owns one native job handle."""

    _rule = None

    def __init__(self, v, r_or_w, h=None, *, eps=REFERENCE_EPS, precision="fp32", seed=0, stream=None,
                 quality_interval=1):
        lib = _native.load()
        if precision not in PRECISIONS:
            raise ValueError("precision must be one of %s" % list(PRECISIONS))
        V = _fortran32(v)
        self.n, self.m = V.shape
        handle = ctypes.c_void_p()
        if h is None:
            r = int(r_or_w)
            st = lib.gpunmf_create_random(self._rule, self.n, self.m, r, _ptr(V), seed, float(eps),
                                          PRECISIONS[precision], stream, ctypes.byref(handle))
        else:
            W = _fortran32(r_or_w)
            H = _fortran32(h)
            if W.shape[0] != self.n or H.shape[1] != self.m or W.shape[1] != H.shape[0]:
                raise ValueError("shapes do not agree: V %s, W %s, H %s" % (V.shape, W.shape, H.shape))
            r = W.shape[1]
            st = lib.gpunmf_create(self._rule, self.n, self.m, r, _ptr(V), _ptr(W), _ptr(H), float(eps),
                                   PRECISIONS[precision], stream, ctypes.byref(handle))
        _native.check(st)
        self.r = r
        self.precision = precision
        self.eps = float(eps)
        self._h = handle
        self._lib = lib
        if quality_interval != 1:
            _native.check(lib.gpunmf_set_quality_interval(self._h, int(quality_interval)))

    # -- reference API ---------------------------------------------------
    def DoIteration(self, updateW=True):
        _native.check(self._lib.gpunmf_iterate(self._h, 1, 1 if updateW else 0))

    def GetW(self):
        out = np.empty((self.n, self.r), dtype=np.float32, order="F")
        _native.check(self._lib.gpunmf_get_w(self._h, _ptr(out)))
        return out

    def GetH(self):
        out = np.empty((self.r, self.m), dtype=np.float32, order="F")
        _native.check(self._lib.gpunmf_get_h(self._h, _ptr(out)))
        return out

    def GetWH(self):
        out = np.empty((self.n, self.m), dtype=np.float32, order="F")
        _native.check(self._lib.gpunmf_get_wh(self._h, _ptr(out)))
        return out

    def QualityImprovement(self):
        out = ctypes.c_float()
        _native.check(self._lib.gpunmf_quality_improvement(self._h, ctypes.byref(out)))
        return out.value

    # -- additions -------------------------------------------------------
    def Iterate(self, iters, updateW=True):
        _native.check(self._lib.gpunmf_iterate(self._h, int(iters), 1 if updateW else 0))

    def SetQualityInterval(self, k):
        """k > 0: sample every k-th iteration (waiting for the previous read-back); 0: never;
        QUALITY_WHEN_READY: the reference's rule (sample when the previous read-back is complete)."""
        _native.check(self._lib.gpunmf_set_quality_interval(self._h, int(k)))

    def Residual(self):
        out = ctypes.c_double()
        _native.check(self._lib.gpunmf_residual_fp64(self._h, ctypes.byref(out)))
        return out.value

    def ObjectiveKL(self):
        out = ctypes.c_double()
        _native.check(self._lib.gpunmf_objective_kl_fp64(self._h, ctypes.byref(out)))
        return out.value

    def Synchronize(self):
        _native.check(self._lib.gpunmf_synchronize(self._h))

    def TimeIterations(self, iters, updateW=True, kernel_timing=False):
        """Device time of `iters` iterations; returns dict(total_ms, kernel_ms, kernel_launches, launches)."""
        tot = ctypes.c_float()
        kms = ctypes.c_float()
        kl = ctypes.c_int()
        al = ctypes.c_int()
        _native.check(self._lib.gpunmf_time_iterations(
            self._h, int(iters), 1 if updateW else 0, ctypes.byref(tot),
            ctypes.byref(kms) if kernel_timing else None, ctypes.byref(kl), ctypes.byref(al)))
        return {"total_ms": tot.value, "kernel_ms": kms.value if kernel_timing else None,
                "kernel_launches": kl.value, "launches": al.value}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gpunmf_destroy(self._h)
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


class NMF_MultiplicativeEuclidianDistance(NMF):
    """Multiplicative updates, Euclidean distance (nmf_multiplicative_euclidian.h:35)."""
    _rule = EUCLIDEAN


class NMF_MultiplicativeDivergence(NMF):
    """Multiplicative updates, Kullback-Leibler divergence (nmf_multiplicative_divergence.h:35)."""
    _rule = DIVERGENCE


class NMF_AdditiveEuclidian(NMF):
    """Additive updates, Euclidean distance (nmf_additive_euclidian.h:35).

    By default it runs exactly what the reference's GPU class runs: that class's
    H step (nmf_additive_euclidian.cpp:37-42) passes (H, deltaH, deltaH2) to the
    multiplicative kernel, which overwrites the deltaH2 workspace and leaves H
    unchanged, so only W is updated.  ``update_h=True`` applies the additive
    step to H as well, as the reference's CPU NMF does (HostNMF.h:152-190).
    """

    def __init__(self, v, r_or_w, h=None, *, update_h=False, **kw):
        self._rule = ADDITIVE_EUCLIDEAN if update_h else ADDITIVE_EUCLIDEAN_FIXED_H
        super().__init__(v, r_or_w, h, **kw)


class NMF_AdditiveDivergence(NMF):
    """Additive updates, Kullback-Leibler divergence (nmf_additive_divergence.h:35)."""
    _rule = ADDITIVE_DIVERGENCE


CLASSES = {EUCLIDEAN: NMF_MultiplicativeEuclidianDistance, DIVERGENCE: NMF_MultiplicativeDivergence,
           ADDITIVE_DIVERGENCE: NMF_AdditiveDivergence}


def make(rule, v, r_or_w, h=None, **kw):
    """The class instance for a rule number (0..4, the gpunmf_rule values)."""
    if rule == ADDITIVE_EUCLIDEAN:
        return NMF_AdditiveEuclidian(v, r_or_w, h, update_h=True, **kw)
    if rule == ADDITIVE_EUCLIDEAN_FIXED_H:
        return NMF_AdditiveEuclidian(v, r_or_w, h, update_h=False, **kw)
    return CLASSES[rule](v, r_or_w, h, **kw)


def footprint_bytes(rule, n, m, r, precision="fp32"):
    return int(_native.load().gpunmf_footprint_bytes(rule, n, m, r, PRECISIONS[precision]))


def device_count():
    return int(_native.load().gpunmf_device_count())


def trim_pool():
    """Hand the library's unused pooled device memory back to the driver (current device)."""
    _native.check(_native.load().gpunmf_trim_pool())
