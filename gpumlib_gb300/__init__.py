"""gpumlib_gb300 — GB300-native multiplicative-update NMF with GPUMLib's class API.

The compute path is the native library libgpunmf.so (hand-written sm_103a
CUDA behind the C ABI of include/gpunmf.h); this package holds its ctypes
binding, a Python mirror of the reference's NMF classes and the synthetic
workload generators.
"""
from .nmf import (NMF, NMF_MultiplicativeDivergence, NMF_MultiplicativeEuclidianDistance, EUCLIDEAN,
                  DIVERGENCE, REFERENCE_EPS, footprint_bytes, device_count)
from ._native import GpuNmfError, load as load_native

__all__ = ["NMF", "NMF_MultiplicativeEuclidianDistance", "NMF_MultiplicativeDivergence", "EUCLIDEAN",
           "DIVERGENCE", "REFERENCE_EPS", "footprint_bytes", "device_count", "GpuNmfError", "load_native"]
