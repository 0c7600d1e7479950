"""The native FacesNMF loader and NMF jobs on the real data set, against the reference's outputs.

The data set (2429 face images, 19 x 19) is staged into oracle/_ref/faces_images by
oracle/build.py wherever the reference tree is present and travels with the checkout;
tests/golden/faces_golden.npz holds what the reference's own code made from it
(tests/golden/make_faces_golden.py): the SHA-256 of V as its loader builds it, and its
HostNMF's W, every 8th column of H and the per-iteration residual at rank 49.

- the GPU loader (decoding + histogram equalisation on the device) gives V bit for bit;
- an FP32 job (the drop-in) from the same seeded W, H gives W and H within 1e-4 relative
  Frobenius of the reference HostNMF after the same iterations (multiplicative Euclidean,
  50 iterations; multiplicative KL, 20), and its residual within 1e-5 relative;
- a BF16 job's residual is within 1e-3 of the reference's.
"""
import hashlib
import os

import numpy as np
import pytest

from conftest import rel
from gpumlib_gb300 import faces, inputs
from oracle import build

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "faces_golden.npz")


@pytest.fixture(scope="module")
def data():
    folder = build.FACES_IMAGES
    if not os.path.isfile(os.path.join(folder, "face00001.pgm")):
        pytest.skip("the FacesNMF data set is not staged (oracle/build.py stages it from the reference tree)")
    return folder, np.load(GOLDEN)


def v_digest(V):
    return hashlib.sha256(np.asfortranarray(V, dtype=np.float32).tobytes(order="F")).hexdigest()


def test_native_loader_matches_reference_loader(gpu, data):
    folder, g = data
    assert faces.scan(folder) == (int(g["count"]), int(g["width"]), int(g["height"]))
    assert v_digest(faces.load(folder, equalize=True)) == str(g["v_sha256"])
    assert v_digest(faces.load(folder, equalize=False)) == str(g["v_plain_sha256"])


@pytest.mark.parametrize("name,rule", [("me", 0), ("kl", 1)])
def test_fp32_job_on_faces_matches_reference_hostnmf(gpu, data, name, rule):
    folder, g = data
    V = faces.load(folder, equalize=True)
    n, m = V.shape
    W, H = inputs.factors(int(g["factor_seed"]), n, m, int(g["rank"]))
    iters = int(g[name + "_iters"])
    with gpu.make(rule, V, W, H, eps=1e-8, precision="fp32", quality_interval=0) as nmf:
        nmf.Iterate(iters)
        Wg, Hg, res = nmf.GetW(), nmf.GetH(), nmf.Residual()
    stride = int(g["h_stride"])
    assert rel(Wg, g[name + "_W"]) <= 1e-4
    assert rel(Hg[:, ::stride], g[name + "_H_cols"]) <= 1e-4
    assert abs(res - g[name + "_resid"][-1]) <= 1e-5 * g[name + "_resid"][-1]


def test_bf16_job_on_faces_reaches_reference_residual(gpu, data):
    folder, g = data
    V = faces.load(folder, equalize=True)
    n, m = V.shape
    W, H = inputs.factors(int(g["factor_seed"]), n, m, int(g["rank"]))
    with gpu.make(0, V, W, H, eps=1e-8, precision="bf16", quality_interval=0) as nmf:
        nmf.Iterate(int(g["me_iters"]))
        res = nmf.Residual()
    assert abs(res - g["me_resid"][-1]) <= 1e-3
