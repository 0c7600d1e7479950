"""Generate tests/golden/hostnmf_golden.npz from the reference's own CPU NMF.

Run in a container that holds the reference tree (it builds
oracle/_ref/libhostnmf_ref.so from src/examples/FacesNMF/HostNMF.h there):

    python tests/golden/make_golden.py

Every case's inputs come from the counter-based generator in
gpumlib_gb300/inputs.py (V from seed `vseed`, W then H from seed `fseed`, each
+1e-4), so only seeds and shapes are stored; the outputs are the reference
HostNMF's W and H after `iters` iterations with its hard-coded epsilon 1e-8
(HostNMF.h:83,110,125,142), plus the relative Frobenius residual after every
iteration.  Cases with `zero_rows` / `zero_cols` zero those rows/columns of V
before running (epsilon-guard edge cases); `sparse` keeps only every k-th
value of V (zeros elsewhere, for the KL ratio).
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from gpumlib_gb300 import inputs  # noqa: E402

CASES = [
    # name, rule, n, m, r, iters, updateW, vseed, fseed, extras
    ("me_1024x512_r16", 0, 1024, 512, 16, 200, True, 0, 1, {}),
    ("me_odd_37x23_r3", 0, 37, 23, 3, 25, True, 11, 12, {}),
    ("me_noW_50x40_r4", 0, 50, 40, 4, 10, False, 13, 14, {}),
    ("me_r1_64x32", 0, 64, 32, 1, 20, True, 15, 16, {}),
    ("me_zeros_32x24_r4", 0, 32, 24, 4, 10, True, 17, 18, {"zero_rows": [3, 17], "zero_cols": [0, 5]}),
    ("me_tall_300x20_r7", 0, 300, 20, 7, 30, True, 19, 20, {}),
    ("kl_256x128_r8", 1, 256, 128, 8, 30, True, 21, 22, {}),
    ("kl_odd_33x17_r5", 1, 33, 17, 5, 15, True, 23, 24, {}),
    ("kl_noW_40x30_r3", 1, 40, 30, 3, 10, False, 25, 26, {}),
    ("kl_sparse_48x40_r4", 1, 48, 40, 4, 10, True, 27, 28, {"sparse": 7}),
    ("kl_wide_20x160_r6", 1, 20, 160, 6, 12, True, 29, 30, {}),
    # additive rules (HostNMF.h:152-233)
    ("ae_200x150_r6", 2, 200, 150, 6, 15, True, 31, 32, {}),
    ("ae_odd_37x23_r3", 2, 37, 23, 3, 10, True, 33, 34, {}),
    ("ae_noW_50x40_r4", 2, 50, 40, 4, 8, False, 35, 36, {}),
    ("ad_256x128_r8", 3, 256, 128, 8, 15, True, 37, 38, {}),
    ("ad_odd_33x17_r5", 3, 33, 17, 5, 10, True, 39, 40, {}),
    ("ad_noW_40x30_r3", 3, 40, 30, 3, 8, False, 41, 42, {}),
]


def case_inputs(case):
    name, rule, n, m, r, iters, updateW, vseed, fseed, extras = case
    V = inputs.uniform_matrix(vseed, n, m)
    if "zero_rows" in extras:
        V[extras["zero_rows"], :] = 0.0
    if "zero_cols" in extras:
        V[:, extras["zero_cols"]] = 0.0
    if "sparse" in extras:
        k = extras["sparse"]
        flat = V.reshape(-1, order="F")
        mask = (np.arange(flat.size) % k) != 0
        flat[mask] = 0.0
        V = np.asfortranarray(flat.reshape(m, n).T)
    W, H = inputs.factors(fseed, n, m, r)
    return V, W, H


def main():
    if oracle.ref() is None:
        sys.exit("the reference tree is not available here; cannot build its HostNMF")
    arrays = {}
    meta = []
    for case in CASES:
        name, rule, n, m, r, iters, updateW, vseed, fseed, extras = case
        V, W, H = case_inputs(case)
        Wo, Ho, res = oracle.reference_run(rule, V, W, H, iters, updateW=updateW, residuals=True)
        arrays[name + "/W"] = Wo
        arrays[name + "/H"] = Ho
        arrays[name + "/resid"] = res
        meta.append(dict(name=name, rule=rule, n=n, m=m, r=r, iters=iters, updateW=updateW, vseed=vseed,
                         fseed=fseed, extras=extras))
        print("%-22s final residual %.6e" % (name, res[-1]))
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hostnmf_golden.npz")
    np.savez_compressed(out, **arrays)
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
