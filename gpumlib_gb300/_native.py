"""ctypes binding of the native library libgpunmf.so (the C ABI of include/gpunmf.h).

The library is built in-tree by gpumlib_gb300._build.build().  There is no
fallback: if the library is missing or fails to load, loading raises.
"""
import ctypes
import os

from . import _build

c_float_p = ctypes.POINTER(ctypes.c_float)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_int_p = ctypes.POINTER(ctypes.c_int)


class Dim3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_uint), ("y", ctypes.c_uint), ("z", ctypes.c_uint)]


# (name, restype, argtypes) of every symbol declared in include/gpunmf.h
SIGNATURES = [
    ("gpunmf_last_error", ctypes.c_char_p, []),
    ("gpunmf_version", ctypes.c_char_p, []),
    ("gpunmf_device_count", ctypes.c_int, []),
    ("gpunmf_create", ctypes.c_int, [ctypes.c_int] * 4 + [ctypes.c_void_p] * 3 +
     [ctypes.c_float, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    ("gpunmf_create_random", ctypes.c_int, [ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_ulonglong,
     ctypes.c_float, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    ("gpunmf_create_device", ctypes.c_int, [ctypes.c_int] * 4 + [ctypes.c_void_p] * 3 +
     [ctypes.c_float, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    ("gpunmf_destroy", ctypes.c_int, [ctypes.c_void_p]),
    ("gpunmf_iterate", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    ("gpunmf_set_quality_interval", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    ("gpunmf_set_wait_limit_cycles", ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong]),
    ("gpunmf_inject_missing_arrival", ctypes.c_int, [ctypes.c_void_p]),
    ("gpunmf_set_grid_limit", ctypes.c_int, [ctypes.c_int]),
    ("gpunmf_quality_improvement", ctypes.c_int, [ctypes.c_void_p, c_float_p]),
    ("gpunmf_residual_fp64", ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    ("gpunmf_objective_kl_fp64", ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    ("gpunmf_residual_fp64_noalloc", ctypes.c_int, [ctypes.c_int] * 3 + [ctypes.c_void_p] * 5),
    ("gpunmf_get_w", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    ("gpunmf_get_h", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    ("gpunmf_get_wh", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    ("gpunmf_device_factors", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                                              ctypes.POINTER(ctypes.c_void_p)]),
    ("gpunmf_synchronize", ctypes.c_int, [ctypes.c_void_p]),
    ("gpunmf_info", ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p, c_float_p]),
    ("gpunmf_footprint_bytes", ctypes.c_size_t, [ctypes.c_int] * 5),
    ("gpunmf_trim_pool", ctypes.c_int, []),
    ("gpunmf_fill_uniform", None, [ctypes.c_ulonglong, ctypes.c_ulonglong, ctypes.c_size_t, ctypes.c_void_p]),
    ("gpunmf_host_alloc", ctypes.c_void_p, [ctypes.c_size_t]),
    ("gpunmf_host_free", None, [ctypes.c_void_p]),
    ("gpunmf_time_iterations", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, c_float_p,
                                               c_float_p, c_int_p, c_int_p]),
    # batched small factorisations
    ("gpunmf_batch_create", ctypes.c_int, [ctypes.c_int] + [ctypes.c_void_p] * 6 + [ctypes.c_float,
                                           ctypes.POINTER(ctypes.c_void_p)]),
    ("gpunmf_batch_destroy", ctypes.c_int, [ctypes.c_void_p]),
    ("gpunmf_batch_run", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    ("gpunmf_batch_synchronize", ctypes.c_int, [ctypes.c_void_p]),
    ("gpunmf_batch_time", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_float_p]),
    ("gpunmf_batch_get", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    ("gpunmf_batch_residuals", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    ("gpunmf_batch_configs", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    ("gpunmf_batch_set_config", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    ("gpunmf_batch_commit", ctypes.c_int, [ctypes.c_void_p]),
    ("gpunmf_batch_reset_factors", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    # serving
    ("gpunmf_server_create", ctypes.c_int, [ctypes.c_int, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_void_p)]),
    ("gpunmf_server_submit", ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong] + [ctypes.c_int] * 4 +
     [ctypes.c_ulonglong, ctypes.c_float]),
    ("gpunmf_server_set_grid_policy", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    ("gpunmf_server_poll", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    ("gpunmf_server_fetch", ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p]),
    ("gpunmf_server_drain", ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    ("gpunmf_server_stats", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong),
                                           ctypes.POINTER(ctypes.c_longlong), c_int_p, c_int_p,
                                           ctypes.POINTER(ctypes.c_size_t)]),
    ("gpunmf_server_clock", ctypes.c_double, [ctypes.c_void_p]),
    ("gpunmf_server_destroy", ctypes.c_int, [ctypes.c_void_p]),
    ("gpunmf_server_generate", ctypes.c_int, [ctypes.c_int] * 3 + [ctypes.c_ulonglong, ctypes.c_float] +
     [ctypes.c_void_p] * 4),
    ("gpunmf_grouped_train", ctypes.c_int,
     [ctypes.c_int] * 5 + [ctypes.c_void_p] * 3 + [ctypes.c_float, ctypes.c_int, ctypes.c_float, ctypes.c_int,
                                                    ctypes.c_void_p]),
    ("gpunmf_faces_scan", ctypes.c_int, [ctypes.c_char_p] + [ctypes.c_void_p] * 3),
    ("gpunmf_faces_load", ctypes.c_int, [ctypes.c_char_p] + [ctypes.c_int] * 5 + [ctypes.c_void_p] * 2),
    ("gpunmf_faces_load_device", ctypes.c_int, [ctypes.c_char_p] + [ctypes.c_int] * 5 + [ctypes.c_void_p] * 3),
    ("gpunmf_save_csv", ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    ("gpunmf_save_csv_device", ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_void_p]),
    ("gpumlib_cuda_nmf_multiplicative_euclidean_update_matrix", ctypes.c_int,
     [ctypes.c_uint, ctypes.c_uint, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    ("gpumlib_cuda_nmf_multiplicative_divergence_update_matrix_w", ctypes.c_int,
     [Dim3, Dim3] + [ctypes.c_void_p] * 5 + [ctypes.c_int] * 3),
    ("gpumlib_cuda_nmf_multiplicative_divergence_update_matrix_h", ctypes.c_int,
     [Dim3, Dim3] + [ctypes.c_void_p] * 5 + [ctypes.c_int] * 3),
    ("gpumlib_cuda_nmf_additive_euclidean_update_matrix", ctypes.c_int,
     [ctypes.c_uint, ctypes.c_uint, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    ("gpumlib_cuda_nmf_additive_divergence_update_matrix_w", ctypes.c_int,
     [Dim3, Dim3] + [ctypes.c_void_p] * 5 + [ctypes.c_int] * 3),
    ("gpumlib_cuda_nmf_additive_divergence_update_matrix_h", ctypes.c_int,
     [Dim3, Dim3] + [ctypes.c_void_p] * 5 + [ctypes.c_int] * 3),
    ("gpumlib_nmf_sum_w", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    ("gpumlib_nmf_sum_h", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    ("gpumlib_nmf_quality", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_void_p]),
]

_lib = None


def lib_path():
    return _build.LIB


def load():
    """Load (once) and return the native library; raises if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError("native library %s is not built; call __graft_entry__.build() "
                           "(or gpumlib_gb300._build.build())" % path)
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def add_signatures(extra):
    """Register further signatures (batch/serve modules) on the loaded library."""
    lib = load()
    for name, res, args in extra:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    SIGNATURES.extend(extra)
    return lib


STATUS = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "NOMEM", 4: "UNSUPPORTED", 5: "NO_DEVICE", 6: "TIMEOUT",
          7: "REJECTED"}


class GpuNmfError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("gpunmf error %s (%d): %s" % (STATUS.get(status, "?"), status, msg))
        self.status = status


def last_error():
    return load().gpunmf_last_error().decode(errors="replace")


def check(status):
    if status != 0:
        lib = load()
        msg = lib.gpunmf_last_error().decode(errors="replace")
        raise GpuNmfError(status, msg)
    return status
