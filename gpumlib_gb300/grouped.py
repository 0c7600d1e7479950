"""Grouped training over the C ABI: FacesNMF's TrainUsingGroups
(src/examples/FacesNMF/FacesNMFDlg.cpp:582-656) as one batched job.

    W, H, iterations = train_using_groups(V, W, H, group, tol)

V (n x m) is cut into floor(m / group) blocks of `group` consecutive columns;
each block is factorised with rank floor(r / blocks) until its quality
improvement drops below ``tol`` (the reference's test) or ``max_iters``.
Block s starts from W[:, s*rs:(s+1)*rs] and the diagonal block
H[s*rs:(s+1)*rs, s*group:(s+1)*group] of the given factors (the reference
draws fresh random factors for every block).  The rule numbers are those of
``gpumlib_gb300.nmf`` (0..4).
"""
import ctypes

import numpy as np

from . import _native
from .nmf import EUCLIDEAN, PRECISIONS, REFERENCE_EPS


def train_using_groups(V, W, H, group, tol, rule=EUCLIDEAN, max_iters=100000, eps=REFERENCE_EPS,
                       precision="fp32"):
    V = np.asfortranarray(V, dtype=np.float32)
    W = np.array(W, dtype=np.float32, order="F", copy=True)
    H = np.array(H, dtype=np.float32, order="F", copy=True)
    n, m = V.shape
    r = W.shape[1]
    if W.shape[0] != n or H.shape != (r, m):
        raise ValueError("shapes do not agree: V %s, W %s, H %s" % (V.shape, W.shape, H.shape))
    blocks = m // int(group) if group > 0 else 0
    iters = np.zeros(max(blocks, 1), dtype=np.int32)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    _native.check(_native.load().gpunmf_grouped_train(
        int(rule), n, m, r, int(group), p(V), p(W), p(H), float(tol), int(max_iters), float(eps),
        PRECISIONS[precision], p(iters)))
    return W, H, iters[:blocks].tolist()
