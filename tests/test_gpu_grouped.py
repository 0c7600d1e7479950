"""Grouped training (FacesNMFDlg.cpp:582-656, TrainUsingGroups) against the oracle's restatement.

The multiplicative Euclidean rule in FP32 runs every block inside one persistent batched launch
that samples the quality and applies the reference's stopping test itself; the other rules run one
engine job per block.  Checks: the block layout of W and H (zeros off the diagonal blocks, columns
outside the blocks unchanged), iteration counts (the quality is a float sum, so a block whose
improvement lands within rounding of tol may stop one iteration apart), and W, H against the
oracle run for the GPU's own iteration counts (FP32 bound 1e-4).
"""
import numpy as np
import pytest

import oracle
from conftest import rel
from gpumlib_gb300 import inputs

pytestmark = pytest.mark.gpu


def data(n, m, r, seed):
    V = inputs.lowrank_gamma(n, m, 8, 2.0, 0.5, seed=seed)
    V = np.asfortranarray(V / V.max())
    W, H = inputs.factors(seed + 10, n, m, r)
    return V, W, H


def check_layout(W0, H0, Wg, Hg, group, blocks, rs):
    assert np.array_equal(Wg[:, blocks * rs:], W0[:, blocks * rs:]), "W columns outside the blocks changed"
    assert np.array_equal(Hg[:, blocks * group:], H0[:, blocks * group:]), "H columns outside the blocks changed"
    for s in range(blocks):
        cols = Hg[:, s * group:(s + 1) * group]
        off = np.delete(cols, np.s_[s * rs:(s + 1) * rs], axis=0)
        assert np.all(off == 0.0), "H outside the diagonal block is not zero"


def compare(gpu, rule, n, m, r, group, tol, seed, precision="fp32", max_iters=5000, slack=1):
    V, W, H = data(n, m, r, seed)
    blocks, rs = m // group, r // (m // group)
    Wg, Hg, its = gpu.train_using_groups(V, W, H, group, tol, rule=rule, max_iters=max_iters,
                                         precision=precision)
    _, _, its_o, _ = oracle.grouped_run(rule, V, W, H, group, tol, max_iters)
    assert len(its) == blocks
    assert all(abs(a - b) <= slack for a, b in zip(its, its_o)), (its, its_o)
    Wo, Ho, _, _ = oracle.grouped_run(rule, V, W, H, group, tol, max_iters, iters_per_block=its)
    check_layout(W, H, Wg, Hg, group, blocks, rs)
    return V, W, H, Wg, Hg, Wo, Ho, its


@pytest.mark.parametrize("shape", [(361, 420, 49, 50), (200, 300, 24, 50), (64, 97, 5, 19)])
def test_grouped_euclidean_batched(gpu, shape):
    n, m, r, group = shape
    _, _, _, Wg, Hg, Wo, Ho, its = compare(gpu, 0, n, m, r, group, 0.01, seed=n, slack=0)
    assert rel(Wg, Wo) <= 1e-4 and rel(Hg, Ho) <= 1e-4


def test_grouped_euclidean_batched_runs_to_max_iters(gpu):
    """A tol no improvement goes below: every block runs max_iters iterations in the batched launch."""
    n, m, r, group = 300, 256, 32, 32
    V, W, H = data(n, m, r, 5)
    Wg, Hg, its = gpu.train_using_groups(V, W, H, group, -3.0e38, max_iters=80)
    assert its == [80] * 8
    Wo, Ho, _, _ = oracle.grouped_run(0, V, W, H, group, -3.0e38, 80)
    assert rel(Wg.astype(np.float64) @ Hg, Wo.astype(np.float64) @ Ho) <= 1e-4
    assert rel(Wg, Wo) <= 1e-4 and rel(Hg, Ho) <= 1e-4


@pytest.mark.parametrize("rule", [1, 3])
def test_grouped_kl_jobs(gpu, rule):
    _, _, _, Wg, Hg, Wo, Ho, its = compare(gpu, rule, 200, 300, 24, 50, 0.01, seed=2)
    assert min(its) > 50
    assert rel(Wg, Wo) <= 1e-4 and rel(Hg, Ho) <= 1e-4


@pytest.mark.parametrize("rule", [2, 4])
def test_grouped_additive_euclidean_jobs(gpu, rule):
    V, W, H, Wg, Hg, Wo, Ho, its = compare(gpu, rule, 150, 160, 12, 40, 0.01, seed=3)
    assert rel(Wg, Wo) <= 1e-4 and rel(Hg, Ho) <= 1e-4
    if rule == 4:  # the reference GPU class's form: each block's H is its starting block
        for s in range(4):
            assert np.array_equal(Hg[s * 3:(s + 1) * 3, s * 40:(s + 1) * 40], H[s * 3:(s + 1) * 3, s * 40:(s + 1) * 40])


def test_grouped_bf16_jobs(gpu):
    """BF16 blocks run as jobs.  The per-iteration quality improvements near a stop are ~1e-5 of the
    quality, below what BF16 products resolve, so a tol-based BF16 stop comes earlier than FP32's;
    with the same iteration counts the BF16 factors track the FP32 ones."""
    n, m, r, group = 256, 384, 48, 64
    V, W, H = data(n, m, r, 7)
    Wf, Hf, itf = gpu.train_using_groups(V, W, H, group, -3.0e38, rule=1, max_iters=40)
    Wb, Hb, itb = gpu.train_using_groups(V, W, H, group, -3.0e38, rule=1, max_iters=40, precision="bf16")
    assert itf == itb == [40] * 6
    check_layout(W, H, Wb, Hb, group, 6, 8)
    assert rel(Wb.astype(np.float64) @ Hb, Wf.astype(np.float64) @ Hf) <= 1e-2
    _, _, its = gpu.train_using_groups(V, W, H, group, 0.3, rule=1, precision="bf16")
    assert all(4 <= k <= 5000 for k in its)


def test_grouped_rejects_bad_shapes(gpu):
    V, W, H = data(40, 30, 4, 9)
    with pytest.raises(gpu.GpuNmfError):
        gpu.train_using_groups(V, W, H, 31, 0.01)      # group > m
    with pytest.raises(gpu.GpuNmfError):
        gpu.train_using_groups(V, W, H, 5, 0.01)       # 6 blocks need r >= 6
