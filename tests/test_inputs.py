"""The seeded synthetic workloads (gpumlib_gb300/inputs.py): the counter-based uniform generator
against an independent restatement of its formula, its offset/chunk invariance and matrix layout,
the project-written normal / gamma / Poisson draws (per-element counters: a draw depends only on
its element; their distributions against the exact ones), digests that pin the generated bytes,
and the shapes and value distributions each workload states."""
import hashlib
import math

import numpy as np
import pytest

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


def splitmix_draw(key, k, draw):
    """Draw `draw` of element k of stream `key`, in plain Python integers: the top 52 bits of
    splitmix64(key + (k 2^16 + draw + 1) golden), plus half a step, times 2^-52."""
    z = (key + (k * 65536 + draw + 1) * 0x9E3779B97F4A7C15) & MASK
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
    z ^= z >> 31
    return ((z >> 12) + 0.5) / 4503599627370496.0


def test_draws_match_formula_and_stay_inside_the_interval():
    key = inputs._stream_key(77, 3)
    idx = np.array([0, 1, 5, 2**30 + 3], dtype=np.uint64)
    for draw in (0, 1, 17, 65535):
        got = inputs._draw(key, idx, draw)
        want = [splitmix_draw(int(key), int(k), draw) for k in idx]
        assert got.tolist() == want
    u = inputs._draw(key, np.arange(200_000, dtype=np.uint64), 0)
    assert 0.0 < u.min() and u.max() < 1.0
    assert inputs._stream_key(77, 3) != inputs._stream_key(77, 4) != inputs._key(77)


def test_draws_depend_only_on_their_element():
    """Any subset, in any order, gives the same values as the whole range (rejection loops
    included): what makes the workloads independent of chunking."""
    key = inputs._stream_key(5, 1)
    full_idx = np.arange(20_000, dtype=np.uint64)
    sub = np.array([19_999, 3, 7_000, 11, 4_242], dtype=np.uint64)
    g = inputs.gamma_draws(key, full_idx, 0.3, 1.0)
    assert np.array_equal(inputs.gamma_draws(key, sub, 0.3, 1.0), g[sub.astype(np.int64)])
    z = inputs.normal_draws(key, full_idx)
    assert np.array_equal(inputs.normal_draws(key, sub), z[sub.astype(np.int64)])
    lam = np.linspace(0.0, 60.0, full_idx.size)
    p = inputs.poisson_draws(key, full_idx, lam)
    assert np.array_equal(inputs.poisson_draws(key, sub, lam[sub.astype(np.int64)]), p[sub.astype(np.int64)])


@pytest.mark.parametrize("shape", [0.3, 1.0, 2.0, 7.5])
def test_gamma_draws_distribution(shape):
    scipy_stats = pytest.importorskip("scipy.stats")
    g = inputs.gamma_draws(inputs._stream_key(11, 2), np.arange(200_000, dtype=np.uint64), shape, 0.5)
    assert g.min() > 0.0
    assert scipy_stats.kstest(g, scipy_stats.gamma(shape, scale=0.5).cdf).pvalue > 1e-3


def test_normal_draws_distribution():
    scipy_stats = pytest.importorskip("scipy.stats")
    z = inputs.normal_draws(inputs._stream_key(12, 3), np.arange(200_000, dtype=np.uint64))
    assert scipy_stats.kstest(z, scipy_stats.norm.cdf).pvalue > 1e-3


@pytest.mark.parametrize("lam", [0.0, 0.5, 3.0, 9.99, 10.0, 11.5, 57.0, 400.0])
def test_poisson_draws_distribution(lam):
    """Inversion below lam = 10, PTRS from 10 on: chi-square against the exact probabilities."""
    scipy_stats = pytest.importorskip("scipy.stats")
    count = 200_000
    p = inputs.poisson_draws(inputs._stream_key(13, 1), np.arange(count, dtype=np.uint64), np.full(count, lam))
    assert np.array_equal(p, np.round(p)) and p.min() >= 0.0
    if lam == 0.0:
        assert p.max() == 0.0
        return
    lo, hi = max(0, int(lam - 5 * math.sqrt(lam))), int(lam + 5 * math.sqrt(lam)) + 1
    ks = np.arange(lo, hi + 1)
    obs = np.concatenate([[(p < lo).sum()], [(p == k).sum() for k in ks], [(p > hi).sum()]]).astype(float)
    exp = count * np.concatenate([[scipy_stats.poisson.cdf(lo - 1, lam)], scipy_stats.poisson.pmf(ks, lam),
                                  [scipy_stats.poisson.sf(hi, lam)]])
    use = exp > 5.0
    chi = float(((obs[use] - exp[use]) ** 2 / exp[use]).sum())
    assert scipy_stats.chi2.sf(chi, int(use.sum()) - 1) > 1e-3


def test_generated_bytes_are_pinned():
    """Digests of small workloads made here: the generator's bytes do not move with a library's
    version (any change to the formulas, the draw numbering or the streams shows here)."""
    def digest(a):
        return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]
    trace = inputs.serving_trace(rate=2000.0, duration=0.05)
    cols = np.array([(j["t"], j["n"], j["m"], j["r"], j["rule"]) for j in trace], dtype=np.float64)
    assert digest(inputs.lowrank_gamma(64, 48, 8, 2.0, 0.5, seed=2)) == "69a6248e57b9ec9e"
    assert digest(inputs.kl_counts(n=256, m=128, r=8)["V"]) == "a721ce70783af839"
    assert digest(np.array(inputs.batched_shapes(16), dtype=np.int64)) == "5ba1bf2c67b1afe8"
    assert len(trace) == 112 and digest(cols) == "c7fd8c1c76f5d16d"
