"""Generate tests/golden/faces_golden.npz from the reference's own FacesNMF code on its data set.

Run in a container that holds the reference tree:

    python tests/golden/make_faces_golden.py

It builds two libraries from the reference's sources (oracle/build.py):
the image loader (FolderHasImages / LoadImage, FacesNMFDlg.cpp:313-347,409-472)
and the CPU NMF (HostNMF.h).  The data set is the reference's 2429 19 x 19 face
images (src/examples/FacesNMF/images), so V is 361 x 2429; the rank is the
dialog's NMF_RANK = 49 (Definitions.h:29) and epsilon HostNMF's 1e-8.

Stored (no pixel data): SHA-256 of the image files and of V in both loader
modes (histogram equalisation on, the dialog's default at FacesNMFDlg.cpp:138,
and off), V's column sums, and for each rule the reference HostNMF's W, every
8th column of H and the relative residual after every iteration, from W and H
drawn by gpumlib_gb300.inputs.factors(FACTOR_SEED, ...).
"""
import ctypes
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import build  # noqa: E402
from gpumlib_gb300 import inputs  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "faces_golden.npz")
RANK = 49
FACTOR_SEED = 49
H_STRIDE = 8
RUNS = [("me", 0, 50), ("kl", 1, 20)]   # name, HostNMF method, iterations


def files_digest(folder, count):
    h = hashlib.sha256()
    for k in range(1, count + 1):
        with open(os.path.join(folder, "face%05d.pgm" % k), "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def v_digest(V):
    return hashlib.sha256(np.asfortranarray(V, dtype=np.float32).tobytes(order="F")).hexdigest()


def reference_load(lib, folder, count, width, height, equalize):
    V = np.zeros((width * height, count), dtype=np.float32, order="F")
    ok = np.zeros(count, dtype=np.int32)
    failed = lib.ref_faces_load(os.fsencode(folder), count, width, height, 1 if equalize else 0,
                                V.ctypes.data_as(ctypes.c_void_p), ok.ctypes.data_as(ctypes.c_void_p))
    if failed:
        raise RuntimeError("%d images failed to load" % failed)
    return V


def main():
    lib_path = build.build_ref_faces()
    if lib_path is None or build.build_ref() is None:
        raise SystemExit("the reference tree is needed (set GPUNMF_REFERENCE_ROOT)")
    images = build.stage_faces_images()
    lib = ctypes.CDLL(lib_path)
    folder = build.backslash_folder(images, os.path.join(build.REF_DIR, "faces_backslash"))
    c, w, h = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    if lib.ref_faces_scan(os.fsencode(folder), ctypes.byref(c), ctypes.byref(w), ctypes.byref(h)) != 1:
        raise SystemExit("FolderHasImages found no images")
    count, width, height = c.value, w.value, h.value
    V = reference_load(lib, folder, count, width, height, True)
    V_plain = reference_load(lib, folder, count, width, height, False)
    n, m = V.shape
    W0, H0 = inputs.factors(FACTOR_SEED, n, m, RANK)
    out = {
        "count": np.int32(count), "width": np.int32(width), "height": np.int32(height),
        "rank": np.int32(RANK), "factor_seed": np.int32(FACTOR_SEED), "h_stride": np.int32(H_STRIDE),
        "files_sha256": np.array(files_digest(images, count)),
        "v_sha256": np.array(v_digest(V)), "v_plain_sha256": np.array(v_digest(V_plain)),
        "v_colsum": V.astype(np.float64).sum(axis=0),
    }
    for name, method, iters in RUNS:
        Wr, Hr, resid = oracle.reference_run(method, V, W0.copy(order="F"), H0.copy(order="F"), iters,
                                             updateW=True, residuals=True)
        out[name + "_iters"] = np.int32(iters)
        out[name + "_W"] = np.asarray(Wr, dtype=np.float32)
        out[name + "_H_cols"] = np.ascontiguousarray(np.asarray(Hr, dtype=np.float32)[:, ::H_STRIDE])
        out[name + "_resid"] = np.asarray(resid, dtype=np.float64)
        print(name, iters, "final residual %.6f" % resid[-1])
    np.savez_compressed(OUT, **out)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
