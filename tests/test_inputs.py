"""The seeded synthetic workloads (gpumlib_gb300/inputs.py): the counter-based uniform generator
against an independent restatement of its formula, its offset/chunk invariance and matrix layout,
and the shapes and value distributions each workload states."""
import math

import numpy as np

from gpumlib_gb300 import inputs

MASK = (1 << 64) - 1


def splitmix_uniform(seed, k):
    """Element k of the stream, in plain Python integers: the top 24 bits of
    splitmix64(key(seed) + (k + 1) * golden) times 2^-24."""
    key = (seed * 0xD1B54A32D192ED03 + 0x8CB92BA72F3D8DD7) & MASK
    z = (key + (k + 1) * 0x9E3779B97F4A7C15) & MASK
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
    z ^= z >> 31
    return (z >> 40) / 16777216.0


def test_uniform_matches_formula():
    for seed in (0, 1, 3, 12345, 2**40 + 7):
        got = inputs.uniform(seed, 64)
        want = np.array([splitmix_uniform(seed, k) for k in range(64)], dtype=np.float32)
        assert np.array_equal(got, want)


def test_uniform_offset_chunk_and_range():
    a = inputs.uniform(9, 5000)
    assert np.array_equal(inputs.uniform(9, 300, offset=4700), a[4700:])
    assert np.array_equal(inputs.uniform(9, 5000, chunk=7), a)
    assert a.dtype == np.float32 and a.min() >= 0.0 and a.max() < 1.0
    assert abs(float(a.mean()) - 0.5) < 0.02
    assert not np.array_equal(a, inputs.uniform(10, 5000))


def test_matrices_are_column_major_streams():
    M = inputs.uniform_matrix(4, 6, 5, add=0.25)
    assert M.shape == (6, 5) and M.flags.f_contiguous
    flat = inputs.uniform(4, 30) + np.float32(0.25)
    assert M[2, 3] == flat[3 * 6 + 2]
    W, H = inputs.factors(8, 10, 7, 3)
    assert np.array_equal(W, inputs.uniform_matrix(8, 10, 3, 0, 1e-4))
    assert np.array_equal(H, inputs.uniform_matrix(8, 3, 7, 30, 1e-4))  # H continues W's stream
    assert W.min() >= 1e-4 and H.min() >= 1e-4


def test_lowrank_gamma_mean_and_noise():
    V = inputs.lowrank_gamma(256, 192, 64, 2.0, 0.5, seed=2)
    assert V.shape == (256, 192) and V.dtype == np.float32 and V.flags.f_contiguous
    assert V.min() > 0.0
    # E[A B] = k * (shape * scale)^2 = 64; |N(0, 0.01)| adds ~0.008
    assert abs(float(V.mean()) - 64.0) < 4.0
    assert np.array_equal(V, inputs.lowrank_gamma(256, 192, 64, 2.0, 0.5, seed=2))


def test_kl_counts_are_counts():
    d = inputs.kl_counts(n=512, m=256, r=16)
    V = d["V"]
    assert V.shape == (512, 256) and d["W"].shape == (512, 16) and d["H"].shape == (16, 256)
    assert np.array_equal(V, np.round(V)) and V.min() >= 0
    # mean lambda = 128 * 0.3^2 = 11.5: almost no zeros
    assert abs(float(V.mean()) - 11.52) < 2.5
    assert float((V == 0).mean()) < 0.05
    sparse = inputs.kl_counts(n=512, m=256, r=16, lam_scale=0.01)["V"]
    assert 0.6 < float((sparse == 0).mean()) < 0.99
    assert d["rule"] == 1 and d["eps"] == 1e-9


def test_batched_shapes_ranges_and_instances():
    shapes = inputs.batched_shapes(200)
    assert len(shapes) == 200
    for n, m, r in shapes:
        assert 32 <= n <= 1024 and 32 <= m <= 512 and r in (4, 8, 16, 32)
    inst = inputs.batched_instance(5)
    assert (inst["n"], inst["m"], inst["r"]) == shapes[5]
    assert inst["V"].shape == (inst["n"], inst["m"]) and inst["W"].min() >= 1e-4


def test_serving_trace_rate_and_mix():
    jobs = inputs.serving_trace(rate=2000.0, duration=2.0)
    ts = [j["t"] for j in jobs]
    assert ts == sorted(ts) and ts[-1] < 2.0
    assert abs(len(jobs) - 4000) < 4 * math.sqrt(4000)
    assert all(64 <= j["n"] <= 4096 and 64 <= j["m"] <= 4096 and 8 <= j["r"] <= 64 for j in jobs)
    kl = sum(j["rule"] for j in jobs) / len(jobs)
    assert abs(kl - 0.3) < 0.03
    assert len({j["seed"] for j in jobs}) == len(jobs)
    V, W, H = inputs.serving_job_data(jobs[0])
    assert V.shape == (jobs[0]["n"], jobs[0]["m"]) and W.shape == (jobs[0]["n"], jobs[0]["r"])
    assert V.min() >= 0.0
