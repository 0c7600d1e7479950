"""FacesNMF data-set I/O: the PGM loader with histogram equalisation (FacesNMFDlg.cpp:409-472), the
image probe (:309-347) and the CSV format of Save (:913-924).

CPU tests pin the oracle's restatement on hand-checkable images; GPU tests compare the native loader
(decoding and equalisation on the device) and the native CSV writer with the oracle, bit for bit and
byte for byte, on seeded synthetic image folders laid out like the data set (19x19 P5 files).
"""
import os

import numpy as np
import pytest

from oracle import faces as ofaces


def make_folder(path, count, width=19, height=19, seed=0, extras=None):
    rng = np.random.Generator(np.random.PCG64(seed))
    os.makedirs(path, exist_ok=True)
    for k in range(1, count + 1):
        px = rng.integers(0, 256, size=width * height, dtype=np.uint8)
        if extras and k in extras:
            kind = extras[k]
            if kind == "constant":
                px[:] = 77
            elif kind == "two":
                px[:] = 10
                px[::3] = 200
            elif kind == "bad_magic":
                ofaces.write_pgm(face(path, k), px, width, height, magic=b"P2")
                continue
            elif kind == "bad_size":
                ofaces.write_pgm(face(path, k), px[:-width], width, height - 1)
                continue
            elif kind == "bad_max":
                ofaces.write_pgm(face(path, k), px, width, height, maxval=65535)
                continue
        ofaces.write_pgm(face(path, k), px, width, height)
    return path


def face(folder, k):
    return ofaces.face_path(folder, k)


# ----------------------------------------------------------------------------- CPU: the oracle
def test_oracle_plain_and_offset(tmp_path):
    px = np.arange(6, dtype=np.uint8) * 40
    ofaces.write_pgm(str(tmp_path / "face00001.pgm"), px, 3, 2)
    v_pgm = ofaces.load_image(str(tmp_path / "face00001.pgm"), 3, 2, False, reference_offset=False)
    assert np.array_equal(v_pgm, (px.astype(np.float32) / np.float32(255)))
    v_ref = ofaces.load_image(str(tmp_path / "face00001.pgm"), 3, 2, False, reference_offset=True)
    # the reference's read starts at the header's final '\n' (byte 10): pixel 0 is it, the last pixel is lost
    assert v_ref[0] == np.float32(10) / np.float32(255)
    assert np.array_equal(v_ref[1:], v_pgm[:-1])


def test_oracle_equalisation_by_hand(tmp_path):
    px = np.array([0, 0, 50, 50, 50, 255], dtype=np.uint8)   # counts 2, 3, 1 -> cum 2, 5, 6; cdfmin 2
    ofaces.write_pgm(str(tmp_path / "face00001.pgm"), px, 6, 1)
    v = ofaces.load_image(str(tmp_path / "face00001.pgm"), 6, 1, True, reference_offset=False)
    exp = np.array([0, 0, 3 / 4, 3 / 4, 3 / 4, 1], dtype=np.float32)
    assert np.array_equal(v, exp)


def test_oracle_scan_probe(tmp_path):
    folder = make_folder(str(tmp_path / "f"), 37)
    assert ofaces.scan(folder) == (37, 19, 19)


def test_oracle_csv_format():
    M = np.array([[0.5, 1.0], [0.25, 2.0 ** -25], [0.0, 12345.6875]], dtype=np.float32)
    text = ofaces.csv_text(M)
    lines = text.split("\n")
    assert len(lines) == 3 and lines[2] == ""              # one line per column
    assert lines[0] == "0.50000000000000000000,0.25000000000000000000,0.00000000000000000000"
    # 2^-25 = 0.0000000298023223876953125: the 21st decimal is 5 followed by nonzero digits, so it rounds up
    assert lines[1] == "1.00000000000000000000,0.00000002980232238770,12345.68750000000000000000"


# ----------------------------------------------------------------------------- GPU: the native path
@pytest.mark.gpu
@pytest.mark.parametrize("equalize", [False, True])
@pytest.mark.parametrize("reference_offset", [True, False])
def test_loader_matches_oracle(gpu, tmp_path, equalize, reference_offset):
    folder = make_folder(str(tmp_path / "faces"), 300, seed=1, extras={5: "constant", 9: "two"})
    count, w, h = gpu.faces.scan(folder)
    assert (count, w, h) == ofaces.scan(folder) == (300, 19, 19)
    V = gpu.faces.load(folder, equalize=equalize, reference_offset=reference_offset)
    Vo, failed = ofaces.load(folder, count, w, h, equalize, reference_offset)
    assert not failed
    assert V.shape == (361, 300)
    assert np.array_equal(V, Vo, equal_nan=True)          # a constant image equalises to 0/0 = NaN in both
    if equalize and not reference_offset:
        assert np.isnan(V[:, 4]).all()                    # image 5 is constant
    if equalize and reference_offset:
        # the header's '\n' joins the constant pixels: two values, so no NaN
        assert not np.isnan(V[:, 4]).any() and V[0, 4] == 0.0


@pytest.mark.gpu
def test_loader_reports_bad_images(gpu, tmp_path):
    folder = make_folder(str(tmp_path / "bad"), 40, seed=2, extras={3: "bad_magic", 7: "bad_size", 11: "bad_max"})
    with pytest.raises(gpu.faces.LoadError) as ei:
        gpu.faces.load(folder, equalize=True)
    err = ei.value
    assert err.failed == 3
    Vo, failed = ofaces.load(folder, 40, 19, 19, True)
    assert failed == [2, 6, 10]
    assert np.array_equal(err.V, Vo)                      # failed columns are zero, the rest loaded


@pytest.mark.gpu
def test_loader_wide_images(gpu, tmp_path):
    folder = make_folder(str(tmp_path / "wide"), 17, width=300, height=257, seed=3)
    V = gpu.faces.load(folder, equalize=True)
    Vo, _ = ofaces.load(folder, 17, 300, 257, True)
    assert np.array_equal(V, Vo)


@pytest.mark.gpu
def test_csv_matches_oracle(gpu, tmp_path):
    rng = np.random.Generator(np.random.PCG64(4))
    M = rng.random((361, 49), dtype=np.float32)
    M[0, 0] = 0.0
    M[1, 0] = np.float32(1e-30)
    M[2, 0] = np.float32(3.4e10)
    M[3, 0] = -np.float32(0.125)
    M[4, 0] = np.nextafter(np.float32(0), np.float32(1))   # smallest subnormal
    path = str(tmp_path / "W.csv")
    gpu.faces.save_csv(path, M)
    assert open(path).read() == ofaces.csv_text(M)
    H = rng.random((49, 1000), dtype=np.float32)
    gpu.faces.save_csv(str(tmp_path / "H.csv"), H)
    assert open(str(tmp_path / "H.csv")).read() == ofaces.csv_text(H)


@pytest.mark.gpu
def test_faces_end_to_end(gpu, tmp_path):
    """Load -> NMF (rank 49, the FacesNMF default) -> CSV, against the oracle pipeline."""
    import oracle
    from gpumlib_gb300 import inputs
    folder = make_folder(str(tmp_path / "e2e"), 120, seed=5)
    V = gpu.faces.load(folder, equalize=True)
    W, H = inputs.factors(6, 361, 120, 49)
    with gpu.NMF_MultiplicativeEuclidianDistance(V, W, H) as nmf:
        nmf.Iterate(20)
        Wg, Hg = nmf.GetW(), nmf.GetH()
    Vo, _ = ofaces.load(folder, 120, 19, 19, True)
    Wo, Ho = oracle.hostnmf_run(0, Vo, W, H, 20, eps=1e-8, nthreads=4)
    from conftest import rel
    assert rel(Wg.astype(np.float64) @ Hg, Wo.astype(np.float64) @ Ho) <= 1e-4
    gpu.faces.save_csv(str(tmp_path / "W.csv"), Wg)
    assert open(str(tmp_path / "W.csv")).read() == ofaces.csv_text(Wg)
