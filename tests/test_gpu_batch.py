"""Batched small factorisations (one persistent, graph-captured launch).

Every instance must match the float oracle of the reference rule
(HostNMF.h:64-114 order of updates) within the drop-in bound: 1e-4 relative
Frobenius on W H after the same iterations.
"""
import numpy as np
import pytest

import oracle
from conftest import rel
from gpumlib_gb300 import batch as gb
from gpumlib_gb300 import inputs

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 1), (5, 3, 2), (33, 17, 3), (64, 64, 4), (100, 40, 5), (37, 300, 8), (257, 129, 13),
          (512, 96, 16), (1024, 512, 32), (300, 500, 20), (32, 32, 32), (700, 33, 7), (45, 1000, 31),
          (128, 128, 1), (600, 600, 24), (1000, 37, 16)]


def make_instances(shapes, seed0=500):
    out = []
    for k, (n, m, r) in enumerate(shapes):
        V = inputs.uniform_matrix(seed0 + k, n, m)
        W, H = inputs.factors(seed0 + 100 + k, n, m, r)
        out.append(dict(V=V, W=W, H=H))
    return out


def test_batch_matches_oracle(gpu):
    insts = make_instances(SHAPES)
    iters = 12
    with gb.Batch(insts) as b:
        b.run(iters)
        b.synchronize()
        res = b.residuals()
        for k, d in enumerate(insts):
            Wg, Hg = b.get(k)
            Wo, Ho = oracle.hostnmf_run(0, d["V"], d["W"], d["H"], iters, eps=1e-8)
            assert rel(Wg.astype(np.float64) @ Hg, Wo.astype(np.float64) @ Ho) <= 1e-4, SHAPES[k]
            assert abs(res[k] - oracle.residual(d["V"], Wg, Hg)) <= 1e-5, SHAPES[k]


def test_batch_configs_agree(gpu):
    """Every tile configuration of a rank class computes the same factorisation."""
    shapes = [(300, 200, 4), (300, 200, 8), (300, 200, 16), (300, 200, 32), (77, 513, 6), (513, 77, 30)]
    insts = make_instances(shapes, seed0=600)
    ranks = gb.configs()
    results = {}
    with gb.Batch(insts) as b:
        for c, rc in enumerate(ranks):
            b.reset_factors()
            for k, (n, m, r) in enumerate(shapes):
                if gb.rank_class(r) == rc:
                    b.set_config(k, c)
            b.commit()
            b.run(6)
            for k, (n, m, r) in enumerate(shapes):
                if gb.rank_class(r) == rc:
                    results.setdefault(k, []).append(b.get(k))
    for k, outs in results.items():
        W0, H0 = outs[0]
        for W1, H1 in outs[1:]:
            assert rel(W1.astype(np.float64) @ H1, W0.astype(np.float64) @ H0) <= 1e-5


def test_graph_replay_continues(gpu):
    insts = make_instances(SHAPES[:8], seed0=700)
    with gb.Batch(insts) as a, gb.Batch(insts) as b:
        a.run(5)
        a.run(5)
        b.run(10)
        for k in range(len(insts)):
            Wa, Ha = a.get(k)
            Wb, Hb = b.get(k)
            assert np.array_equal(Wa, Wb) and np.array_equal(Ha, Hb)


def test_autotune_assigns_matching_configs(gpu):
    insts = [inputs.batched_instance(i) for i in range(48)]
    ranks = gb.configs()
    with gb.Batch(insts) as b:
        table = gb.autotune(b, insts, sample=16, iters=2)
        assert table
        for k, (n, m, r) in enumerate(b.shapes):
            assert b.cfg[k] is not None and ranks[b.cfg[k]] == gb.rank_class(r)
        b.run(4)
        b.synchronize()
        res = b.residuals()
    assert np.all(np.isfinite(res)) and np.all(res < 1.0)


def test_batch_rejects_large_rank(gpu):
    d = make_instances([(20, 20, 40)])[0]
    with pytest.raises(gpu.GpuNmfError):
        gb.Batch([d])
