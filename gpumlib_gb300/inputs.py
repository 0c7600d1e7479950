"""Seeded synthetic workloads for the NMF engine.

The reference ships no benchmark data (its only dataset is the FacesNMF image
folder), so every workload is synthetic with the shapes and value
distributions below.

* ``uniform(seed, count, offset)`` is a counter-based generator: element k
  is the top 24 bits of splitmix64(key(seed) + (offset+k+1)*0x9E3779B97F4A7C15)
  times 2^-24.  It is pure integer arithmetic, so it gives the same bits on
  every machine and in the C++ engine (gpunmf_create_random uses the same
  formula).
* Gamma, normal and Poisson draws, the batched instances' shapes and the serving
  trace come from the same splitmix64 counters through distributions written
  here (``gamma_draws``, ``normal_draws``, ``poisson_draws``): element k of a
  stream owns its own counters, so a draw depends only on (seed, stream, k)
  and no library generator (nor its version) is involved.  Streams of one seed
  are told apart by a byte in the key's top bits (``_stream_key``).

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


# ---------------------------------------------------------------------------
# distributions over the counter-based generator
# ---------------------------------------------------------------------------
_STEP52 = 1.0 / 4503599627370496.0  # 2^-52
_DRAWS = 1 << 16                    # counters per element of a stream


def _mix(z):
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def _draw(key, idx, draw):
    """float64 uniforms strictly inside (0, 1): draw number `draw` (< 2^16) of elements `idx`
    (uint64 array) of stream `key`, the top 52 bits of splitmix64(key + (idx 2^16 + draw + 1)
    * golden) plus half a step."""
    with np.errstate(over="ignore"):
        z = _mix(key + (idx * np.uint64(_DRAWS) + np.uint64(draw + 1)) * _GOLDEN)
    return ((z >> np.uint64(12)).astype(np.float64) + 0.5) * _STEP52


def _normal(key, idx, draw):
    """Standard normals by Box-Muller (its cosine branch) from draws `draw` and `draw + 1`."""
    u1, u2 = _draw(key, idx, draw), _draw(key, idx, draw + 1)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def normal_draws(key, idx):
    """N(0, 1) for elements `idx` of stream `key` (float64)."""
    return _normal(key, np.asarray(idx, dtype=np.uint64), 0)


def gamma_draws(key, idx, shape, scale=1.0, max_attempts=64):
    """Gamma(shape, scale) for elements `idx` of stream `key` (float64), by Marsaglia and Tsang's
    method (ACM Trans. Math. Software 26(3), 2000): with d = a - 1/3 and c = 1 / sqrt(9 d), attempt t
    of an element takes a normal x (draws 3t, 3t + 1) and a uniform u (draw 3t + 2); with
    v = (1 + c x)^3 > 0 it accepts d v when u < 1 - 0.0331 x^4 or log u < x^2 / 2 + d (1 - v + log v).
    For shape < 1 it draws Gamma(shape + 1) and multiplies by u^(1 / shape) (the paper's boost), u
    from the element's last draw."""
    idx = np.asarray(idx, dtype=np.uint64)
    a = shape if shape >= 1.0 else shape + 1.0
    d = a - 1.0 / 3.0
    c = 1.0 / math.sqrt(9.0 * d)
    out = np.empty(idx.size, dtype=np.float64)
    pend = np.arange(idx.size)
    for t in range(max_attempts):
        if pend.size == 0:
            break
        el = idx[pend]
        x = _normal(key, el, 3 * t)
        u = _draw(key, el, 3 * t + 2)
        v = 1.0 + c * x
        pos = v > 0.0
        v = np.where(pos, v * v * v, 1.0)
        with np.errstate(divide="ignore", invalid="ignore"):
            ok = pos & ((u < 1.0 - 0.0331 * (x * x) * (x * x)) |
                        (np.log(u) < 0.5 * x * x + d * (1.0 - v + np.log(v))))
        out[pend[ok]] = d * v[ok]
        pend = pend[~ok]
    if pend.size:
        raise RuntimeError("gamma_draws: %d elements not accepted in %d attempts" % (pend.size, max_attempts))
    if shape < 1.0:
        out *= _draw(key, idx, _DRAWS - 1) ** (1.0 / shape)
    return out * scale


def poisson_draws(key, idx, lam, max_attempts=64, max_search=100):
    """Poisson(lam) for elements `idx` of stream `key` (lam >= 0 per element; float64 counts).
    lam < 10: inversion by sequential search (one uniform, draw 0; the probabilities by their
    recurrence p(k) = p(k - 1) lam / k from exp(-lam)).  lam >= 10: Hormann's transformed rejection
    with squeeze, PTRS (Insurance: Mathematics and Economics 12, 1993), attempt t taking draws 2t and
    2t + 1."""
    idx = np.asarray(idx, dtype=np.uint64).ravel()
    lam = np.asarray(lam, dtype=np.float64).ravel()
    out = np.empty(idx.size, dtype=np.float64)
    small = np.flatnonzero(lam < 10.0)
    if small.size:
        u = _draw(key, idx[small], 0)
        ls = lam[small]
        p = np.exp(-ls)
        cdf = p.copy()
        k = np.zeros(small.size)
        res = np.zeros(small.size)
        pos = np.arange(small.size)
        for _ in range(max_search):  # cut there: P(k >= 100) < 1e-50 for lam < 10
            keep = u > cdf  # the searches still going, compacted each pass
            u, ls, p, cdf, k, pos = u[keep], ls[keep], p[keep], cdf[keep], k[keep], pos[keep]
            if pos.size == 0:
                break
            k += 1.0
            p *= ls / k
            cdf += p
            res[pos] = k
        out[small] = res
    big = np.flatnonzero(lam >= 10.0)
    if big.size:
        lb = lam[big]
        slam, loglam = np.sqrt(lb), np.log(lb)
        b = 0.931 + 2.53 * slam
        a = -0.059 + 0.02483 * b
        invalpha = 1.1239 + 1.1328 / (b - 3.4)
        vr = 0.9277 - 3.6224 / (b - 2.0)
        pend = np.arange(big.size)
        for t in range(max_attempts):
            if pend.size == 0:
                break
            el = idx[big[pend]]
            U = _draw(key, el, 2 * t) - 0.5
            V = _draw(key, el, 2 * t + 1)
            us = 0.5 - np.abs(U)
            ap, bp = a[pend], b[pend]
            k = np.floor((2.0 * ap / us + bp) * U + lb[pend] + 0.43)
            quick = (us >= 0.07) & (V <= vr[pend])
            test = ~quick & ~((k < 0.0) | ((us < 0.013) & (V > us)))
            ok = quick.copy()
            if test.any():
                kt = k[test]
                ks, inv = np.unique(kt, return_inverse=True)
                lgk = np.array([math.lgamma(float(q) + 1.0) for q in ks])[inv.ravel()]
                lhs = np.log(V[test]) + np.log(invalpha[pend[test]]) - np.log(ap[test] / (us[test] * us[test]) + bp[test])
                rhs = -lb[pend[test]] + kt * loglam[pend[test]] - lgk
                ok[np.flatnonzero(test)[lhs <= rhs]] = True
            out[big[pend[ok]]] = k[ok]
            pend = pend[~ok]
        if pend.size:
            raise RuntimeError("poisson_draws: %d elements not accepted in %d attempts" % (pend.size, max_attempts))
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


def _gamma_matrix(seed, stream, rows, cols, shape, scale):
    """rows x cols Gamma(shape, scale) draws (float64, column-major element order)."""
    g = gamma_draws(_stream_key(seed, stream), np.arange(rows * cols, dtype=np.uint64), shape, scale)
    return colmajor(g, rows, cols)


def lowrank_gamma(n, m, k, shape, scale, seed, noise_sd=0.01):
    """A (n x k) @ B (k x m) with Gamma(shape, scale) entries (streams 1 and 2 of `seed`), plus
    |N(0, noise_sd)| (stream 3, element by column-major index); float32."""
    A = _gamma_matrix(seed, 1, n, k, shape, scale)
    B = _gamma_matrix(seed, 2, k, m, shape, scale)
    V = np.asfortranarray((A @ B).astype(np.float32))
    if noise_sd:
        nkey = _stream_key(seed, 3)
        cols_per = max(1, (1 << 24) // max(1, n))
        for c0 in range(0, m, cols_per):
            c1 = min(m, c0 + cols_per)
            z = normal_draws(nkey, np.arange(c0 * n, c1 * n, dtype=np.uint64))
            V[:, c0:c1] += colmajor(np.abs(noise_sd * z).astype(np.float32), n, c1 - c0)
    return V


def large_euclidean(n=8192, m=8192, r=64):
    """Large Euclidean MU: V = A B + |N(0,0.01)|, A n x 64, B 64 x m ~ Gamma(2, 0.5) (seed 2);
    W, H U[0,1)+1e-4 (seed 3); r = 64; 500 iterations."""
    V = lowrank_gamma(n, m, 64, 2.0, 0.5, seed=2)
    W, H = factors(3, n, m, r)
    return dict(V=V, W=W, H=H, r=r, iters=500, eps=1e-9, rule=0)


def kl_counts(n=16384, m=4096, r=128, lam_scale=1.0):
    """KL MU on counts: V ~ Poisson(P Q) (stream 3 of seed 4, element by column-major index),
    P n x 128, Q 128 x m ~ Gamma(0.3, 1) (streams 1 and 2 of seed 4); W, H U[0,1)+1e-4 (seed 5);
    r = 128; 300 iterations; eps 1e-9."""
    P = _gamma_matrix(4, 1, n, 128, 0.3, 1.0)
    Q = _gamma_matrix(4, 2, 128, m, 0.3, 1.0)
    pkey = _stream_key(4, 3)
    V = np.empty((n, m), dtype=np.float32, order="F")
    step = max(1, (1 << 24) // n)
    for c0 in range(0, m, step):
        c1 = min(m, c0 + step)
        lam = np.asfortranarray((P @ Q[:, c0:c1]) * lam_scale)
        counts = poisson_draws(pkey, np.arange(c0 * n, c1 * n, dtype=np.uint64), lam.ravel(order="F"))
        V[:, c0:c1] = colmajor(counts.astype(np.float32), n, c1 - c0)
    W, H = factors(5, n, m, r)
    return dict(V=V, W=W, H=H, r=r, iters=300, eps=1e-9, rule=1)


def _batched_shape(i):
    """(n, m, r) of batched instance i: draws 0-2 of element 0 of stream 5 of seed 1000 + i."""
    key, z = _stream_key(1000 + i, 5), np.zeros(1, dtype=np.uint64)
    m = 32 + int(_draw(key, z, 0)[0] * 481)
    n = 32 + int(_draw(key, z, 1)[0] * 993)
    r = (4, 8, 16, 32)[int(_draw(key, z, 2)[0] * 4)]
    return n, m, r


def batched_instance(i):
    """Instance i of the batched workload (seed 1000+i): m ~ U{32..512}, n ~ U{32..1024},
    r ~ {4,8,16,32}; V U[0,1) float32, then W, H U[0,1)+1e-4, one counter stream of the seed."""
    n, m, r = _batched_shape(i)
    V = uniform_matrix(1000 + i, n, m)
    W = uniform_matrix(1000 + i, n, r, n * m, 1e-4)
    H = uniform_matrix(1000 + i, r, m, n * m + n * r, 1e-4)
    return dict(V=V, W=W, H=H, n=n, m=m, r=r)


def batched_shapes(count=4096):
    """(n, m, r) of the first `count` batched instances, without drawing V."""
    return [_batched_shape(i) for i in range(count)]


def serving_trace(rate=2000.0, duration=60.0, seed=7, lo=64, hi=4096, rmin=8, rmax=64, kl_frac=0.3):
    """Poisson arrivals; per job: n, m log-uniform in [lo, hi], r ~ U{rmin..rmax},
    rule KL with probability kl_frac; returns a list of dicts (without V)."""
    # job j: draws 0-4 of element j of stream 6 of `seed` (gap, n, m, r, rule)
    key = _stream_key(seed, 6)
    llo, lhi = math.log(lo), math.log(hi)
    t = 0.0
    jobs = []
    block = 4096
    while True:
        j = np.arange(len(jobs), len(jobs) + block, dtype=np.uint64)
        gap = -np.log(_draw(key, j, 0)) / rate
        n = np.rint(np.exp(llo + _draw(key, j, 1) * (lhi - llo)))
        m = np.rint(np.exp(llo + _draw(key, j, 2) * (lhi - llo)))
        r = rmin + np.floor(_draw(key, j, 3) * (rmax - rmin + 1))
        kl = _draw(key, j, 4) < kl_frac
        for q in range(block):
            t += float(gap[q])
            if t >= duration:
                return jobs
            jobs.append(dict(id=len(jobs), t=t, n=int(n[q]), m=int(m[q]), r=int(r[q]), rule=1 if kl[q] else 0,
                             seed=10_000_000 + len(jobs)))


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
