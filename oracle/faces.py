"""CPU restatement of the FacesNMF data-set I/O, for the tests only.

TEST INFRASTRUCTURE ONLY: the product never imports this module.

load_image follows src/examples/FacesNMF/FacesNMFDlg.cpp:409-472 (LoadImage):
the header is read with istream >> semantics, the pixel block starts right
after the max-gray-value digits (the reference's read() begins at the
whitespace byte that ends the header) unless reference_offset is False, and
the histogram equalisation is the reference's float arithmetic:
cumulative counts, cdfmin = the first nonzero one, (cum - cdfmin) /
(pixels - cdfmin).  scan follows FolderHasImages (:309-347) and csv_text
follows Save (:913-924) with PRECISION 20 (Definitions.h:31).  Pinned bit for
bit against the reference's own FolderHasImages / LoadImage, compiled from
FacesNMFDlg.cpp with stand-ins for the MFC names (oracle/ref_faces_shim.cpp),
on the whole FacesNMF data set and on edge-case images
(tests/test_faces_real_data.py).  Save is not pinned that way: it writes
through MFC file dialogs.
"""
import os

import numpy as np

_WS = b" \t\n\r\v\f"


def _token(buf, pos):
    while pos < len(buf) and buf[pos] in _WS:
        pos += 1
    start = pos
    while pos < len(buf) and buf[pos] not in _WS:
        pos += 1
    return buf[start:pos], pos


def _integer(buf, pos):
    while pos < len(buf) and buf[pos] in _WS:
        pos += 1
    start = pos
    if pos < len(buf) and buf[pos] in b"+-":
        pos += 1
    d0 = pos
    while pos < len(buf) and 48 <= buf[pos] <= 57:
        pos += 1
    if pos == d0:
        raise ValueError("no integer")
    return int(buf[start:pos]), pos


def face_path(folder, number):
    return os.path.join(folder, "face%05d.pgm" % number)


def load_image(path, width, height, equalize, reference_offset=True):
    """One column of V (float32), or raises ValueError as the reference reports an error."""
    buf = open(path, "rb").read()
    magic, pos = _token(buf, 0)
    if magic != b"P5":
        raise ValueError("Invalid image format")
    w, pos = _integer(buf, pos)
    h, pos = _integer(buf, pos)
    if w != width or h != height:
        raise ValueError("Incorrect image size")
    maxval, pos = _integer(buf, pos)
    if maxval != 255:
        raise ValueError("Check max gray value")
    if not reference_offset and pos < len(buf) and buf[pos] in _WS:
        pos += 1
    pixels = width * height
    if len(buf) < pos + pixels:
        raise ValueError("image data too short")
    px = np.frombuffer(buf[pos:pos + pixels], dtype=np.uint8)
    if not equalize:
        lut = (np.arange(256, dtype=np.float32) / np.float32(255.0)).astype(np.float32)
        return lut[px]
    hist = np.zeros(256, dtype=np.float32)
    np.add.at(hist, px, np.float32(1.0))
    cum = np.cumsum(hist, dtype=np.float32)          # integers < 2^24: exact in float
    i = int(np.argmax(cum != 0))
    cdfmin = cum[i]
    lut = np.zeros(256, dtype=np.float32)
    with np.errstate(invalid="ignore", divide="ignore"):
        lut[i:] = (cum[i:] - cdfmin) / (np.float32(pixels) - cdfmin)
    return lut[px]


def scan(folder):
    """(count, width, height) as FolderHasImages finds them."""
    buf = open(face_path(folder, 1), "rb").read()
    magic, pos = _token(buf, 0)
    if magic != b"P5":
        raise ValueError("Invalid image format")
    w, pos = _integer(buf, pos)
    h, pos = _integer(buf, pos)
    n, inc = 0, 1024
    while True:
        if not os.path.isfile(face_path(folder, n + inc)):
            if inc == 1:
                break
            inc >>= 1
        else:
            n += inc
    return n, w, h


def load(folder, count, width, height, equalize, reference_offset=True):
    """V (pixels x count, float32, column-major) and the list of images that failed (zero columns)."""
    V = np.zeros((width * height, count), dtype=np.float32, order="F")
    failed = []
    for k in range(count):
        try:
            V[:, k] = load_image(face_path(folder, k + 1), width, height, equalize, reference_offset)
        except (ValueError, OSError):
            failed.append(k)
    return V, failed


def csv_text(M):
    """Save(): one line per column, values '%.20f' joined by commas."""
    M = np.asarray(M, dtype=np.float32)
    lines = []
    for c in range(M.shape[1]):
        lines.append(",".join("%.20f" % float(x) for x in M[:, c]))
    return "".join(line + "\n" for line in lines)


def write_pgm(path, pixels, width, height, maxval=255, magic=b"P5"):
    """A P5 file laid out like the data set's (single '\\n' after each header line)."""
    with open(path, "wb") as f:
        f.write(magic + b"\n%d %d\n%d\n" % (width, height, maxval))
        f.write(np.asarray(pixels, dtype=np.uint8).tobytes())
