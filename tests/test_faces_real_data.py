"""The FacesNMF data set itself (2429 face images, 19 x 19, src/examples/FacesNMF/images).

Pins, all bit for bit:
- where the reference tree is present, the reference's own loader (FolderHasImages /
  LoadImage, FacesNMFDlg.cpp:313-347,409-472, compiled from its source by oracle/build.py)
  against the restatement oracle/faces.py, on every image of the data set in both modes
  and on edge-case images (constant image, bad magic, size and max gray value);
- the staged data set (oracle/_ref/faces_images, copied from the reference tree at build
  time) against the digests in tests/golden/faces_golden.npz, which the reference loader
  made (tests/golden/make_faces_golden.py);
- the oracle's float HostNMF on that V against the reference HostNMF's W and H there
  (rank 49, the dialog's NMF_RANK).
Without a reference tree and without the staged images these skip; the GPU side
(tests/test_gpu_faces_real.py) compares the native loader and an FP32 job with the same
golden data.
"""
import ctypes
import hashlib
import os

import numpy as np
import pytest

import oracle
from oracle import build
from oracle import faces as ofaces
from gpumlib_gb300 import inputs
from test_faces_io import make_folder

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "faces_golden.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def v_digest(V):
    return hashlib.sha256(np.asfortranarray(V, dtype=np.float32).tobytes(order="F")).hexdigest()


def staged_images():
    folder = build.FACES_IMAGES
    if not os.path.isfile(os.path.join(folder, "face00001.pgm")):
        pytest.skip("the FacesNMF data set is not staged (oracle/build.py stages it from the reference tree)")
    return folder


@pytest.fixture(scope="module")
def ref_loader():
    path = build.build_ref_faces()
    if path is None:
        pytest.skip("reference tree absent: the reference loader cannot be built")
    return ctypes.CDLL(path)


def ref_load(lib, folder, workdir, count, width, height, equalize):
    bs = build.backslash_folder(folder, workdir)
    V = np.zeros((width * height, count), dtype=np.float32, order="F")
    ok = np.zeros(count, dtype=np.int32)
    lib.ref_faces_load(os.fsencode(bs), count, width, height, 1 if equalize else 0,
                       V.ctypes.data_as(ctypes.c_void_p), ok.ctypes.data_as(ctypes.c_void_p))
    return V, ok


def ref_scan(lib, folder, workdir):
    bs = build.backslash_folder(folder, workdir)
    c, w, h = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    found = lib.ref_faces_scan(os.fsencode(bs), ctypes.byref(c), ctypes.byref(w), ctypes.byref(h))
    return found, c.value, w.value, h.value


@pytest.mark.parametrize("equalize", [True, False], ids=["equalised", "plain"])
def test_reference_loader_matches_oracle_on_data_set(ref_loader, tmp_path, equalize):
    folder = build.stage_faces_images()
    found, count, width, height = ref_scan(ref_loader, folder, str(tmp_path / "bs"))
    assert found == 1 and (count, width, height) == ofaces.scan(folder) == (2429, 19, 19)
    Vr, ok = ref_load(ref_loader, folder, str(tmp_path / "bs"), count, width, height, equalize)
    Vo, failed = ofaces.load(folder, count, width, height, equalize)
    assert ok.all() and failed == []
    assert np.array_equal(Vr.view(np.uint32), Vo.view(np.uint32))


@pytest.mark.parametrize("equalize", [True, False], ids=["equalised", "plain"])
def test_reference_loader_matches_oracle_on_edge_images(ref_loader, tmp_path, equalize):
    extras = {2: "constant", 3: "two", 5: "bad_magic", 6: "bad_size", 8: "bad_max"}
    folder = make_folder(str(tmp_path / "imgs"), 9, seed=7, extras=extras)
    found, count, width, height = ref_scan(ref_loader, folder, str(tmp_path / "bs"))
    assert found == 1 and (count, width, height) == ofaces.scan(folder)
    Vr, ok = ref_load(ref_loader, folder, str(tmp_path / "bs"), count, width, height, equalize)
    Vo, failed = ofaces.load(folder, count, width, height, equalize)
    assert sorted(np.flatnonzero(ok == 0).tolist()) == failed == [4, 5, 7]
    good = ok == 1
    assert np.array_equal(Vr[:, good].view(np.uint32), Vo[:, good].view(np.uint32))
    if equalize:   # the 'constant' image is not constant as read: its pixel 0 is the header's '\n'
        assert Vr[0, 1] == 0.0 and (Vr[1:, 1] == 1.0).all()


def test_staged_data_set_matches_golden_digests(golden):
    folder = staged_images()
    count = int(golden["count"])
    h = hashlib.sha256()
    for k in range(1, count + 1):
        with open(ofaces.face_path(folder, k), "rb") as f:
            h.update(f.read())
    assert h.hexdigest() == str(golden["files_sha256"])
    assert ofaces.scan(folder) == (count, int(golden["width"]), int(golden["height"]))
    V, failed = ofaces.load(folder, count, 19, 19, True)
    assert failed == [] and v_digest(V) == str(golden["v_sha256"])
    np.testing.assert_array_equal(V.astype(np.float64).sum(axis=0), golden["v_colsum"])
    Vp, _ = ofaces.load(folder, count, 19, 19, False)
    assert v_digest(Vp) == str(golden["v_plain_sha256"])


@pytest.mark.parametrize("name,rule", [("me", 0), ("kl", 1)])
def test_oracle_hostnmf_on_faces_matches_reference(golden, name, rule):
    folder = staged_images()
    V, _ = ofaces.load(folder, int(golden["count"]), 19, 19, True)
    n, m = V.shape
    W0, H0 = inputs.factors(int(golden["factor_seed"]), n, m, int(golden["rank"]))
    W, H = oracle.hostnmf_run(rule, V, W0, H0, int(golden[name + "_iters"]), nthreads=os.cpu_count() or 1)
    stride = int(golden["h_stride"])
    assert np.array_equal(W.view(np.uint32), golden[name + "_W"].view(np.uint32))
    assert np.array_equal(np.ascontiguousarray(H[:, ::stride]).view(np.uint32),
                          golden[name + "_H_cols"].view(np.uint32))
