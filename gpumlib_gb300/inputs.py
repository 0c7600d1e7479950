"""Seeded synthetic workloads for the NMF engine.

The reference ships no benchmark data (its only dataset is the FacesNMF image
folder), so every workload is synthetic with the shapes and value
distributions below.

* ``uniform(seed, count, offset)`` is a counter-based generator: element k
  is the top 24 bits of splitmix64(key(seed) + (offset+k+1)*0x9E3779B97F4A7C15)
  times 2^-24.  It is pure integer arithmetic, so it gives the same bits on
  every machine and in the C++ engine (gpunmf_create_random uses the same
  formula).
* Gamma / normal / Poisson draws use numpy's PCG64 generator with the stated
  seed (``numpy.random.Generator(PCG64(seed))``).

Matrices are returned as column-major (Fortran-ordered) float32 arrays; a
"column-major flat index" k of an n x m matrix is u*n + i.
"""
import math

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_MASK = (1 << 64) - 1
_SCALE = np.float32(1.0 / 16777216.0)


def _key(seed):
    return np.uint64((int(seed) * 0xD1B54A32D192ED03 + 0x8CB92BA72F3D8DD7) & _MASK)


def uniform(seed, count, offset=0, chunk=1 << 22):
    """count float32 values in [0, 1) from the counter-based generator."""
    out = np.empty(int(count), dtype=np.float32)
    key = _key(seed)
    with np.errstate(over="ignore"):
        for lo in range(0, int(count), chunk):
            hi = min(int(count), lo + chunk)
            z = np.arange(offset + lo + 1, offset + hi + 1, dtype=np.uint64)
            z = key + z * _GOLDEN
            z = (z ^ (z >> np.uint64(30))) * _M1
            z = (z ^ (z >> np.uint64(27))) * _M2
            z = z ^ (z >> np.uint64(31))
            out[lo:hi] = (z >> np.uint64(40)).astype(np.float32) * _SCALE
    return out


def colmajor(flat, rows, cols):
    """View a column-major flat vector as a (rows, cols) Fortran-ordered array."""
    return np.asfortranarray(flat.reshape(cols, rows).T)


def uniform_matrix(seed, rows, cols, offset=0, add=0.0):
    a = uniform(seed, rows * cols, offset)
    if add:
        a += np.float32(add)
    return colmajor(a, rows, cols)


def factors(seed, n, m, r, add=1e-4):
    """W (n x r) then H (r x m) from one counter stream of `seed`, each + add."""
    W = uniform_matrix(seed, n, r, 0, add)
    H = uniform_matrix(seed, r, m, n * r, add)
    return W, H


# ---------------------------------------------------------------------------
# the five workloads
# ---------------------------------------------------------------------------

def plain_euclidean_1024x512():
    """Plain FP32 Euclidean MU: V 1024x512 U[0,1) (seed 0); W, H U[0,1)+1e-4 (seed 1); r=16."""
    n, m, r = 1024, 512, 16
    V = uniform_matrix(0, n, m)
    W, H = factors(1, n, m, r)
    return dict(V=V, W=W, H=H, r=r, iters=200, eps=1e-9, rule=0)


def lowrank_gamma(n, m, k, shape, scale, seed, noise_sd=0.01):
    """A (n x k) @ B (k x m) with Gamma(shape, scale) entries, plus |N(0, noise_sd)|; float32."""
    g = np.random.Generator(np.random.PCG64(seed))
    A = g.gamma(shape, scale, size=(n, k))
    B = g.gamma(shape, scale, size=(k, m))
    V = np.asfortranarray((A @ B).astype(np.float32))
    if noise_sd:
        rows_per = max(1, (1 << 24) // max(1, n))
        for c0 in range(0, m, rows_per):
            c1 = min(m, c0 + rows_per)
            V[:, c0:c1] += np.abs(g.normal(0.0, noise_sd, size=(n, c1 - c0))).astype(np.float32)
    return V


def large_euclidean(n=8192, m=8192, r=64):
    """Large Euclidean MU: V = A B + |N(0,0.01)|, A n x 64, B 64 x m ~ Gamma(2, 0.5) (seed 2);
    W, H U[0,1)+1e-4 (seed 3); r = 64; 500 iterations."""
    V = lowrank_gamma(n, m, 64, 2.0, 0.5, seed=2)
    W, H = factors(3, n, m, r)
    return dict(V=V, W=W, H=H, r=r, iters=500, eps=1e-9, rule=0)


def kl_counts(n=16384, m=4096, r=128, lam_scale=1.0):
    """KL MU on counts: V ~ Poisson(P Q), P n x 128, Q 128 x m ~ Gamma(0.3, 1) (seed 4);
    W, H U[0,1)+1e-4 (seed 5); r = 128; 300 iterations; eps 1e-9."""
    g = np.random.Generator(np.random.PCG64(4))
    P = g.gamma(0.3, 1.0, size=(n, 128))
    Q = g.gamma(0.3, 1.0, size=(128, m))
    V = np.empty((n, m), dtype=np.float32, order="F")
    step = max(1, (1 << 24) // n)
    for c0 in range(0, m, step):
        c1 = min(m, c0 + step)
        lam = (P @ Q[:, c0:c1]) * lam_scale
        V[:, c0:c1] = g.poisson(lam).astype(np.float32)
    W, H = factors(5, n, m, r)
    return dict(V=V, W=W, H=H, r=r, iters=300, eps=1e-9, rule=1)


def batched_instance(i):
    """Instance i of the batched workload (seed 1000+i): m ~ U{32..512}, n ~ U{32..1024},
    r ~ {4,8,16,32}; V U[0,1) float32; W, H U[0,1)+1e-4 from the same generator."""
    g = np.random.Generator(np.random.PCG64(1000 + i))
    m = int(g.integers(32, 513))
    n = int(g.integers(32, 1025))
    r = int(g.choice([4, 8, 16, 32]))
    V = np.asfortranarray(g.random((n, m), dtype=np.float32))
    W = np.asfortranarray(g.random((n, r), dtype=np.float32) + np.float32(1e-4))
    H = np.asfortranarray(g.random((r, m), dtype=np.float32) + np.float32(1e-4))
    return dict(V=V, W=W, H=H, n=n, m=m, r=r)


def batched_shapes(count=4096):
    """(n, m, r) of the first `count` batched instances, without drawing V."""
    out = []
    for i in range(count):
        g = np.random.Generator(np.random.PCG64(1000 + i))
        m = int(g.integers(32, 513))
        n = int(g.integers(32, 1025))
        r = int(g.choice([4, 8, 16, 32]))
        out.append((n, m, r))
    return out


def serving_trace(rate=2000.0, duration=60.0, seed=7, lo=64, hi=4096, rmin=8, rmax=64, kl_frac=0.3):
    """Poisson arrivals; per job: n, m log-uniform in [lo, hi], r ~ U{rmin..rmax},
    rule KL with probability kl_frac; returns a list of dicts (without V)."""
    g = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    jobs = []
    while True:
        t += g.exponential(1.0 / rate)
        if t >= duration:
            break
        n = int(round(math.exp(g.uniform(math.log(lo), math.log(hi)))))
        m = int(round(math.exp(g.uniform(math.log(lo), math.log(hi)))))
        r = int(g.integers(rmin, rmax + 1))
        rule = 1 if g.random() < kl_frac else 0
        jobs.append(dict(id=len(jobs), t=t, n=n, m=m, r=r, rule=rule, seed=10_000_000 + len(jobs)))
    return jobs


def _stream_key(seed, stream):
    """Key of stream `stream` of a served job's seed: the counter generator's key with the stream
    number in its top byte (the device generator's key schedule)."""
    return np.uint64(int(_key(seed)) ^ (int(stream) << 56))


def _uniform_key(key, count):
    z = np.arange(1, int(count) + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = key + z * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(40)).astype(np.float32) * _SCALE


def serving_job_data(job, noise_sd=0.01):
    """Host twin of the served jobs' device generator: V = A B + |N(0, noise_sd)| with A n x r and
    B r x m uniform[0,1) (streams 0 and 1 of the job seed), the noise by Box-Muller from stream 2
    (element k from uniforms 2k and 2k+1, the first shifted by half a step off zero); W, H
    uniform[0,1) + 1e-4 (streams 3 and 4).  The uniforms are the same bits as on the device; V
    differs from the device's only by float rounding (the product's summation order, log/cos).
    Returns float32 column-major (V, W, H)."""
    n, m, r, seed = job["n"], job["m"], job["r"], job["seed"]
    A = colmajor(_uniform_key(_stream_key(seed, 0), n * r), n, r)
    B = colmajor(_uniform_key(_stream_key(seed, 1), r * m), r, m)
    u = _uniform_key(_stream_key(seed, 2), 2 * n * m).astype(np.float64)
    u1, u2 = u[0::2] + 0.5 / 16777216.0, u[1::2]
    z = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
    noise = colmajor(np.abs(noise_sd * z).astype(np.float32), n, m)
    V = np.asfortranarray((A.astype(np.float64) @ B.astype(np.float64)).astype(np.float32) + noise)
    W = colmajor(_uniform_key(_stream_key(seed, 3), n * r) + np.float32(1e-4), n, r)
    H = colmajor(_uniform_key(_stream_key(seed, 4), r * m) + np.float32(1e-4), r, m)
    return V, W, H
