"""The FacesNMF data set over the C ABI (src/examples/FacesNMF/FacesNMFDlg.cpp).

    count, width, height = scan(folder)                 # FolderHasImages (:309-347)
    V = load(folder, equalize=True)                     # LoadImage (:409-472) for every image
    save_csv("W.csv", nmf.GetW())                        # Save (:913-924)

``load`` decodes and equalises on the GPU and returns a host array
(``gpunmf_faces_load_device`` in the C ABI leaves V in device memory instead,
ready for ``gpunmf_create_device``).
``reference_offset`` (default True) reads the pixel block where the reference
does, one byte early (pixel 0 is the header's final newline, the last pixel is
not read); False reads standard PGM.
"""
import ctypes
import os

import numpy as np

from . import _native


def _b(path):
    return os.fsencode(path)


def scan(folder):
    c, w, h = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _native.check(_native.load().gpunmf_faces_scan(_b(folder), ctypes.byref(c), ctypes.byref(w), ctypes.byref(h)))
    return c.value, w.value, h.value


class LoadError(RuntimeError):
    """Some images failed; ``V`` holds the others (failed columns are zero)."""

    def __init__(self, msg, V, failed):
        super().__init__(msg)
        self.V = V
        self.failed = failed


def load(folder, equalize=False, count=None, reference_offset=True):
    n_img, w, h = scan(folder)
    if count is None:
        count = n_img
    V = np.empty((w * h, count), dtype=np.float32, order="F")
    failed = ctypes.c_int()
    st = _native.load().gpunmf_faces_load(_b(folder), int(count), w, h, 1 if equalize else 0,
                                           1 if reference_offset else 0, V.ctypes.data_as(ctypes.c_void_p),
                                           ctypes.byref(failed))
    if st == 1 and failed.value > 0:
        raise LoadError(_native.last_error(), V, failed.value)
    _native.check(st)
    return V


def save_csv(path, M):
    M = np.asfortranarray(M, dtype=np.float32)
    rows, cols = M.shape
    _native.check(_native.load().gpunmf_save_csv(_b(path), M.ctypes.data_as(ctypes.c_void_p), rows, cols))
