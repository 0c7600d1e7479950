"""gpumlib_gb300 — GB300-native NMF (multiplicative and additive rules) with GPUMLib's class API.

The compute path is the native library libgpunmf.so (hand-written sm_103a
CUDA behind the C ABI of include/gpunmf.h); this package holds its ctypes
binding, a Python mirror of the reference's NMF classes and the synthetic
workload generators.
"""
from .nmf import (NMF, NMF_MultiplicativeDivergence, NMF_MultiplicativeEuclidianDistance, NMF_AdditiveEuclidian,
                  NMF_AdditiveDivergence, EUCLIDEAN, DIVERGENCE, ADDITIVE_EUCLIDEAN, ADDITIVE_DIVERGENCE,
                  ADDITIVE_EUCLIDEAN_FIXED_H, REFERENCE_EPS, QUALITY_WHEN_READY, footprint_bytes, device_count, make, trim_pool)
from ._native import GpuNmfError, load as load_native
from .grouped import train_using_groups
from . import faces

__all__ = ["NMF", "NMF_MultiplicativeEuclidianDistance", "NMF_MultiplicativeDivergence", "NMF_AdditiveEuclidian",
           "NMF_AdditiveDivergence", "EUCLIDEAN", "DIVERGENCE", "ADDITIVE_EUCLIDEAN", "ADDITIVE_DIVERGENCE",
           "ADDITIVE_EUCLIDEAN_FIXED_H", "REFERENCE_EPS", "QUALITY_WHEN_READY", "footprint_bytes", "device_count", "make", "trim_pool",
           "GpuNmfError", "load_native", "train_using_groups", "faces"]
