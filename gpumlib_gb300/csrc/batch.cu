// Batched multiplicative-update NMF: thousands of small, uneven Euclidean
// factorisations in one persistent launch, and FacesNMF's grouped training on
// top of it (end of file).
//
// The reference's nearest equivalent is FacesNMF's grouped training
// (src/examples/FacesNMF/FacesNMFDlg.cpp:582-656), which builds one NMF
// object per group and runs them one after another, each iteration being a
// handful of cuBLAS calls and kernel launches.  Here every CTA is a small
// NMF engine: it takes the next instance from a largest-first work list
// (atomic counter), runs all its iterations itself, and moves on.  Because
// one CTA owns the instance, an iteration needs no grid-wide sync and every
// step is fused:
//   H-step, per chunk of BC columns:  W'V chunk (streaming V), den = G_W H,
//                                     H update, and the chunk's part of H H'
//   W-step, per chunk of BC rows:     V H' chunk (streaming V), den = W G_H,
//                                     W update, and the chunk's part of W'W
// so each iteration reads V exactly twice (from L2: a few hundred instances
// in flight fit in the 129 MB L2) and W, H a few times.  Arithmetic is FP32
// on the CUDA cores, the same rule and order as the plain drop-in path
// (nmf_multiplicative_euclidian.cpp:29-67, nmf_kernels.cu:43-47).
//
// Tile shapes (BC, BI) are template parameters; each instance carries the
// index of the shape an autotuner picked for its (r, size) bucket.
#include <algorithm>
#include <mutex>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "engine.h"
#include "kernels.h"

namespace gpunmf {

struct BatchInst {
    long long v, w, h;  // offsets (floats) into the packed V, W, H buffers
    int n, m, r, cfg;
};

constexpr int kBatchThreads = 256;

// per-instance convergence test (grouped training)
struct BatchStop {
    float tol;
    int *iterations;  // [instances] iterations run
};
constexpr int kBatchSmemFloats = 12288;  // 48 KB

// 4-byte asynchronous global -> shared copy; zero-fills when !valid (src is then not read)
__device__ __forceinline__ void cp_async_f32(float *dst, const float *src, bool valid) {
    const unsigned saddr = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(saddr), "l"(src), "r"(valid ? 4 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}

// ---------------------------------------------------------------------------
// one instance, rank R (padded rank: W, H columns/rows beyond r are zero),
// column/row chunk BC, streaming tile BI.
// ---------------------------------------------------------------------------
template <int R, int BC, int BI>
struct InstanceRunner {
    static constexpr int TU = 4;                               // columns (or rows) per thread
    static constexpr int AG = (R * BC) / (kBatchThreads * TU) >= 1 ? R / ((R * BC) / (kBatchThreads * TU)) : R;
    static constexpr int TA = R / AG;                          // ranks per thread
    static constexpr int UG = kBatchThreads / AG;              // thread groups along the chunk
    static_assert(AG * TA == R && UG * TU == BC, "tile does not cover the chunk");
    static constexpr int GE = (R * R + kBatchThreads - 1) / kBatchThreads;  // Gram entries per thread

    // shared memory carve (floats)
    static constexpr int OFF_G = 0;               // [R][R] current Gram (denominator)
    static constexpr int OFF_V = OFF_G + R * R;   // [BI][BC+4]   V tile
    static constexpr int OFF_F = OFF_V + BI * (BC + 4);  // [BI][R+4] W rows (H-step) or [BI][R+4] H cols (W-step)
    static constexpr int OFF_X = OFF_F + BI * (R + 4);   // [R][BC+4] H chunk (H-step) / W chunk^T (W-step)
    static constexpr int TOTAL = OFF_X + R * (BC + 4);
    static_assert(TOTAL <= kBatchSmemFloats, "shared memory");

    __device__ static void gram_init(float *sG, const float *X, long long ldx, int rows, int r, bool x_is_w,
                                     float *sv) {
        // G = X' X over `rows` (W: X(i,a) = W[a*ldx + i]); computed straight from global (L2)
        const int tid = threadIdx.x;
        float acc[GE];
#pragma unroll
        for (int e = 0; e < GE; e++) acc[e] = 0.f;
        for (int i0 = 0; i0 < rows; i0 += BI) {
            const int nr = min(BI, rows - i0);
            for (int k = tid; k < BI * R; k += kBatchThreads) {
                const int a = k / BI, ii = k % BI;
                const bool ok = a < r && ii < nr;
                cp_async_f32(&sv[ii * (R + 4) + a], ok ? X + (long long)a * ldx + i0 + ii : X, ok);
            }
            cp_async_wait_all();
            __syncthreads();
#pragma unroll
            for (int e = 0; e < GE; e++) {
                const int q = tid + e * kBatchThreads;
                if (q < R * R) {
                    const int a = q / R, b = q % R;
                    float s = acc[e];
                    for (int ii = 0; ii < BI; ii++) s = fmaf(sv[ii * (R + 4) + a], sv[ii * (R + 4) + b], s);
                    acc[e] = s;
                }
            }
            __syncthreads();
        }
        (void)x_is_w;
#pragma unroll
        for (int e = 0; e < GE; e++) {
            const int q = tid + e * kBatchThreads;
            if (q < R * R) sG[q] = acc[e];
        }
        __syncthreads();
    }

    // quality of the current factors, sum V log10(WH + eps) - WH (nmf_kernels_quality.cu:35), as the
    // float the reference reads back; WH is formed tile by tile and never stored.  Same value on
    // every thread.  Uses the V, factor and chunk areas of shared memory, not the Gram.
    __device__ __noinline__ static float quality(const float *__restrict__ V, const float *__restrict__ W,
                                    const float *__restrict__ H, int n, int m, int r, float eps, float *sm) {
        __shared__ double qred[32];
        float *sV = sm + OFF_V, *sF = sm + OFF_F, *sX = sm + OFF_X;
        const int tid = threadIdx.x;
        constexpr int EPT = BI * BC / kBatchThreads;  // tile elements per thread
        static_assert(EPT * kBatchThreads == BI * BC, "tile/threads");
        double t = 0.0;
        for (int c0 = 0; c0 < m; c0 += BC) {
            const int nc = min(BC, m - c0);
            for (int k = tid; k < R * BC; k += kBatchThreads) {
                const int u = k / R, a = k % R;
                const bool ok = a < r && u < nc;
                cp_async_f32(&sX[a * (BC + 4) + u], ok ? H + (long long)(c0 + u) * r + a : H, ok);
            }
            for (int i0 = 0; i0 < n; i0 += BI) {
                const int nr = min(BI, n - i0);
                for (int k = tid; k < BI * BC; k += kBatchThreads) {
                    const int u = k / BI, ii = k % BI;
                    const bool ok = ii < nr && u < nc;
                    cp_async_f32(&sV[ii * (BC + 4) + u], ok ? V + (long long)(c0 + u) * n + i0 + ii : V, ok);
                }
                for (int k = tid; k < BI * R; k += kBatchThreads) {
                    const int a = k / BI, ii = k % BI;
                    const bool ok = a < r && ii < nr;
                    cp_async_f32(&sF[ii * (R + 4) + a], ok ? W + (long long)a * n + i0 + ii : W, ok);
                }
                cp_async_wait_all();
                __syncthreads();
                float part = 0.f;
#pragma unroll 4
                for (int e = 0; e < EPT; e++) {
                    const int q = tid + e * kBatchThreads, ii = q / BC, u = q % BC;
                    float wh = 0.f;
#pragma unroll
                    for (int a = 0; a < R; a++) wh = fmaf(sF[ii * (R + 4) + a], sX[a * (BC + 4) + u], wh);
                    if (ii < nr && u < nc) part += sV[ii * (BC + 4) + u] * log10f(wh + eps) - wh;
                }
                t += (double)part;
                __syncthreads();
            }
        }
        return (float)block_sum(t, qred);
    }

    // kStop: the convergence test of FacesNMF's grouped training (FacesNMFDlg.cpp:605-629) on the
    // lagged quality improvement of nmf_base.h:70-89; without it exactly `iters` iterations run.
    template <bool kStop>
    __device__ __noinline__ static void run(const BatchInst &d, const float *__restrict__ Vall, float *__restrict__ Wall,
                               float *__restrict__ Hall, float eps, int iters, float *sm,
                               const BatchStop &stop, int inst) {
        const int n = d.n, m = d.m, r = d.r;
        const float *V = Vall + d.v;
        float *W = Wall + d.w;
        float *H = Hall + d.h;
        float *sG = sm + OFF_G, *sV = sm + OFF_V, *sF = sm + OFF_F, *sX = sm + OFF_X;
        const int tid = threadIdx.x;
        const int ag = tid % AG, ug = tid / AG;

        gram_init(sG, W, n, n, r, true, sF);  // G = W'W

        // lag state exactly as the host engine keeps it, held by thread 0 in shared memory; the
        // stop decision is taken when the iteration starts (the improvement it reports is known
        // then) and read by every thread after the iteration's last barrier
        struct Lag {
            float value, last, delta, prev;
            int times, stop_after;
        };
        __shared__ Lag lag;
        if (kStop && tid == 0) lag = Lag{0.f, -1.f, 1.f, 1.f, 0, 0};
        int done = iters;
        for (int it = 0; it < iters; it++) {
            if constexpr (kStop) {
                const float q_new = quality(V, W, H, n, m, r, eps, sm);  // contains barriers
                if (tid == 0) {
                    const float q_now = lag.value;
                    if (lag.times++ > 2) lag.delta = q_now - lag.last;
                    else lag.times++;
                    lag.last = q_now;
                    lag.value = q_new;
                    lag.stop_after = 0;
                    if (lag.delta != lag.prev) {
                        if (lag.delta < stop.tol) lag.stop_after = 1;
                        else lag.prev = lag.delta;
                    }
                }
            }
            // ================= H-step =================
            float gacc[GE];
#pragma unroll
            for (int e = 0; e < GE; e++) gacc[e] = 0.f;
            for (int c0 = 0; c0 < m; c0 += BC) {
                const int nc = min(BC, m - c0);
                float acc[TA][TU];
#pragma unroll
                for (int i = 0; i < TA; i++)
#pragma unroll
                    for (int j = 0; j < TU; j++) acc[i][j] = 0.f;
                // numerator W'V for the chunk
                for (int i0 = 0; i0 < n; i0 += BI) {
                    const int nr = min(BI, n - i0);
                    for (int k = tid; k < BI * BC; k += kBatchThreads) {
                        const int u = k / BI, ii = k % BI;
                        const bool ok = ii < nr && u < nc;
                        cp_async_f32(&sV[ii * (BC + 4) + u], ok ? V + (long long)(c0 + u) * n + i0 + ii : V, ok);
                    }
                    for (int k = tid; k < BI * R; k += kBatchThreads) {
                        const int a = k / BI, ii = k % BI;
                        const bool ok = a < r && ii < nr;
                        cp_async_f32(&sF[ii * (R + 4) + a], ok ? W + (long long)a * n + i0 + ii : W, ok);
                    }
                    cp_async_wait_all();
                    __syncthreads();
#pragma unroll 4
                    for (int ii = 0; ii < BI; ii++) {
                        float wv[TA], vv[TU];
#pragma unroll
                        for (int i = 0; i < TA; i++) wv[i] = sF[ii * (R + 4) + ag * TA + i];
#pragma unroll
                        for (int j = 0; j < TU; j++) vv[j] = sV[ii * (BC + 4) + ug * TU + j];
#pragma unroll
                        for (int i = 0; i < TA; i++)
#pragma unroll
                            for (int j = 0; j < TU; j++) acc[i][j] = fmaf(wv[i], vv[j], acc[i][j]);
                    }
                    __syncthreads();
                }
                // H chunk into shared memory
                for (int k = tid; k < R * BC; k += kBatchThreads) {
                    const int u = k / R, a = k % R;
                    const bool ok = a < r && u < nc;
                    cp_async_f32(&sX[a * (BC + 4) + u], ok ? H + (long long)(c0 + u) * r + a : H, ok);
                }
                cp_async_wait_all();
                __syncthreads();
                // den = G H ; H *= num / (den + eps)
                float hn[TA][TU];
#pragma unroll
                for (int i = 0; i < TA; i++)
#pragma unroll
                    for (int j = 0; j < TU; j++) {
                        const int a = ag * TA + i, u = ug * TU + j;
                        float den = 0.f;
                        for (int b = 0; b < R; b++) den = fmaf(sG[a * R + b], sX[b * (BC + 4) + u], den);
                        float h = sX[a * (BC + 4) + u];
                        hn[i][j] = (a < r && u < nc) ? h * (acc[i][j] / (den + eps)) : 0.f;
                    }
                __syncthreads();
#pragma unroll
                for (int i = 0; i < TA; i++)
#pragma unroll
                    for (int j = 0; j < TU; j++) sX[(ag * TA + i) * (BC + 4) + ug * TU + j] = hn[i][j];
                __syncthreads();
                for (int k = tid; k < R * BC; k += kBatchThreads) {
                    const int u = k / R, a = k % R;
                    if (a < r && u < nc) H[(long long)(c0 + u) * r + a] = sX[a * (BC + 4) + u];
                }
                // this chunk's part of H H'
#pragma unroll
                for (int e = 0; e < GE; e++) {
                    const int q = tid + e * kBatchThreads;
                    if (q < R * R) {
                        const int a = q / R, b = q % R;
                        float s = gacc[e];
                        for (int u = 0; u < BC; u++) s = fmaf(sX[a * (BC + 4) + u], sX[b * (BC + 4) + u], s);
                        gacc[e] = s;
                    }
                }
                __syncthreads();
            }
#pragma unroll
            for (int e = 0; e < GE; e++) {
                const int q = tid + e * kBatchThreads;
                if (q < R * R) sG[q] = gacc[e];
            }
            __syncthreads();

            // ================= W-step =================
#pragma unroll
            for (int e = 0; e < GE; e++) gacc[e] = 0.f;
            for (int i0 = 0; i0 < n; i0 += BC) {
                const int nr = min(BC, n - i0);
                float acc[TA][TU];  // (a, row) : a = ag*TA+i, row = ug*TU+j
#pragma unroll
                for (int i = 0; i < TA; i++)
#pragma unroll
                    for (int j = 0; j < TU; j++) acc[i][j] = 0.f;
                for (int u0 = 0; u0 < m; u0 += BI) {
                    const int ncu = min(BI, m - u0);
                    for (int k = tid; k < BI * BC; k += kBatchThreads) {
                        const int uu = k / BC, ii = k % BC;
                        const bool ok = ii < nr && uu < ncu;
                        cp_async_f32(&sV[uu * (BC + 4) + ii], ok ? V + (long long)(u0 + uu) * n + i0 + ii : V, ok);
                    }
                    for (int k = tid; k < BI * R; k += kBatchThreads) {
                        const int uu = k / R, a = k % R;
                        const bool ok = a < r && uu < ncu;
                        cp_async_f32(&sF[uu * (R + 4) + a], ok ? H + (long long)(u0 + uu) * r + a : H, ok);
                    }
                    cp_async_wait_all();
                    __syncthreads();
#pragma unroll 4
                    for (int uu = 0; uu < BI; uu++) {
                        float hv[TA], vv[TU];
#pragma unroll
                        for (int i = 0; i < TA; i++) hv[i] = sF[uu * (R + 4) + ag * TA + i];
#pragma unroll
                        for (int j = 0; j < TU; j++) vv[j] = sV[uu * (BC + 4) + ug * TU + j];
#pragma unroll
                        for (int i = 0; i < TA; i++)
#pragma unroll
                            for (int j = 0; j < TU; j++) acc[i][j] = fmaf(hv[i], vv[j], acc[i][j]);
                    }
                    __syncthreads();
                }
                // W rows of the chunk, transposed into sX[a][row]
                for (int k = tid; k < R * BC; k += kBatchThreads) {
                    const int a = k / BC, ii = k % BC;
                    const bool ok = a < r && ii < nr;
                    cp_async_f32(&sX[a * (BC + 4) + ii], ok ? W + (long long)a * n + i0 + ii : W, ok);
                }
                cp_async_wait_all();
                __syncthreads();
                float wn[TA][TU];
#pragma unroll
                for (int i = 0; i < TA; i++)
#pragma unroll
                    for (int j = 0; j < TU; j++) {
                        const int a = ag * TA + i, row = ug * TU + j;
                        float den = 0.f;
                        for (int b = 0; b < R; b++) den = fmaf(sX[b * (BC + 4) + row], sG[b * R + a], den);
                        float w = sX[a * (BC + 4) + row];
                        wn[i][j] = (a < r && row < nr) ? w * (acc[i][j] / (den + eps)) : 0.f;
                    }
                __syncthreads();
#pragma unroll
                for (int i = 0; i < TA; i++)
#pragma unroll
                    for (int j = 0; j < TU; j++) sX[(ag * TA + i) * (BC + 4) + ug * TU + j] = wn[i][j];
                __syncthreads();
                for (int k = tid; k < R * BC; k += kBatchThreads) {
                    const int a = k / BC, ii = k % BC;
                    if (a < r && ii < nr) W[(long long)a * n + i0 + ii] = sX[a * (BC + 4) + ii];
                }
#pragma unroll
                for (int e = 0; e < GE; e++) {
                    const int q = tid + e * kBatchThreads;
                    if (q < R * R) {
                        const int a = q / R, b = q % R;
                        float s = gacc[e];
                        for (int ii = 0; ii < BC; ii++) s = fmaf(sX[a * (BC + 4) + ii], sX[b * (BC + 4) + ii], s);
                        gacc[e] = s;
                    }
                }
                __syncthreads();
            }
#pragma unroll
            for (int e = 0; e < GE; e++) {
                const int q = tid + e * kBatchThreads;
                if (q < R * R) sG[q] = gacc[e];
            }
            __syncthreads();
            if (kStop && lag.stop_after) {
                done = it + 1;
                break;
            }
        }
        if (kStop && tid == 0) stop.iterations[inst] = done;
    }
};

// tile configurations: (R, BC, BI) per config index
#define GPUNMF_BATCH_CONFIGS(X)  \
    X(0, 4, 256, 32)             \
    X(1, 8, 128, 32)             \
    X(2, 16, 64, 32)             \
    X(3, 32, 32, 32)             \
    X(4, 8, 256, 16)             \
    X(5, 16, 64, 16)             \
    X(6, 32, 32, 64)             \
    X(7, 4, 256, 16)

constexpr int kBatchConfigs = 8;
__host__ __device__ constexpr int batch_cfg_rank(int c) {
    return c == 0 ? 4 : c == 1 ? 8 : c == 2 ? 16 : c == 3 ? 32 : c == 4 ? 8 : c == 5 ? 16 : c == 6 ? 32 : 4;  // config 7: rank 4
}

template <bool kStop>
__global__ void __launch_bounds__(kBatchThreads, 3)
    batch_kernel(const BatchInst *__restrict__ insts, const int *__restrict__ order, int count,
                 int *__restrict__ next, const float *__restrict__ V, float *__restrict__ W, float *__restrict__ H,
                 float eps, int iters, BatchStop stop) {
    extern __shared__ float bsm[];
    __shared__ int s_idx;
    for (;;) {
        if (threadIdx.x == 0) s_idx = atomicAdd(next, 1);
        __syncthreads();
        const int k = s_idx;
        __syncthreads();
        if (k >= count) break;
        const BatchInst d = insts[order[k]];
        switch (d.cfg) {
#define X(C, R, BC, BI) \
    case C: InstanceRunner<R, BC, BI>::template run<kStop>(d, V, W, H, eps, iters, bsm, stop, order[k]); break;
            GPUNMF_BATCH_CONFIGS(X)
#undef X
            default: break;
        }
        __syncthreads();
    }
}

// per-instance relative residual, FP64 accumulation, one CTA per instance
__global__ void batch_residual_kernel(const BatchInst *__restrict__ insts, int count, const float *__restrict__ V,
                                      const float *__restrict__ W, const float *__restrict__ H,
                                      double *__restrict__ out) {
    __shared__ double red[32];
    const int k = blockIdx.x;
    if (k >= count) return;
    const BatchInst d = insts[k];
    const float *v = V + d.v, *w = W + d.w, *h = H + d.h;
    double num = 0.0, den = 0.0;
    const long long total = (long long)d.n * d.m;
    for (long long e = threadIdx.x; e < total; e += blockDim.x) {
        const int i = (int)(e % d.n), u = (int)(e / d.n);
        float wh = 0.f;
        for (int a = 0; a < d.r; a++) wh = fmaf(w[(long long)a * d.n + i], h[(long long)u * d.r + a], wh);
        const double x = v[e], dd = x - (double)wh;
        num += dd * dd;
        den += x * x;
    }
    num = block_sum(num, red);
    den = block_sum(den, red);
    if (threadIdx.x == 0) out[k] = den > 0.0 ? sqrt(num / den) : 0.0;
}

}  // namespace gpunmf

using namespace gpunmf;

// ---------------------------------------------------------------------------
// host side: packed buffers, largest-first order, graph-captured launch
// ---------------------------------------------------------------------------
struct gpunmf_batch {
    int count = 0;
    float eps = 1e-8f;
    std::vector<BatchInst> h_insts;
    BatchInst *d_insts = nullptr;
    int *d_order = nullptr;
    int *d_next = nullptr;
    float *V = nullptr, *W = nullptr, *H = nullptr;
    double *d_res = nullptr;
    long long v_total = 0, w_total = 0, h_total = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graph_iters = -1;
    int grid = 0;
};

static int rank_class(int r) { return r <= 4 ? 4 : r <= 8 ? 8 : r <= 16 ? 16 : r <= 32 ? 32 : 0; }

static int default_cfg(int r) {
    switch (rank_class(r)) {
        case 4: return 0;
        case 8: return 1;
        case 16: return 2;
        case 32: return 3;
    }
    return -1;
}

static size_t batch_smem_bytes(int cfg) {
    switch (cfg) {
#define X(C, R, BC, BI) \
    case C: return (size_t)InstanceRunner<R, BC, BI>::TOTAL * sizeof(float);
        GPUNMF_BATCH_CONFIGS(X)
#undef X
    }
    return 0;
}

static size_t batch_max_smem() {
    size_t mx = 0;
    for (int c = 0; c < kBatchConfigs; c++) mx = std::max(mx, batch_smem_bytes(c));
    return mx;
}

// work estimate for the largest-first order: multiply-adds of one iteration
static double inst_cost(const BatchInst &d) {
    const double n = d.n, m = d.m, R = rank_class(d.r);
    return 2.0 * n * m * R + 2.0 * R * R * (n + m);
}

static void order_largest_first(const std::vector<BatchInst> &in, std::vector<int> &order) {
    order.resize(in.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return inst_cost(in[a]) > inst_cost(in[b]); });
}

static void batch_free(gpunmf_batch *b) {
    if (!b) return;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    void *ptrs[] = {b->d_insts, b->d_order, b->d_next, b->V, b->W, b->H, b->d_res};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

static gpunmf_status batch_upload_order(gpunmf_batch *b) {
    std::vector<int> order;
    order_largest_first(b->h_insts, order);
    GPUNMF_CUDA_TRY(cudaMemcpyAsync(b->d_insts, b->h_insts.data(), sizeof(BatchInst) * b->count,
                                    cudaMemcpyHostToDevice, b->stream));
    GPUNMF_CUDA_TRY(cudaMemcpyAsync(b->d_order, order.data(), sizeof(int) * b->count, cudaMemcpyHostToDevice,
                                    b->stream));
    GPUNMF_CUDA_TRY(cudaStreamSynchronize(b->stream));
    return GPUNMF_OK;
}

static gpunmf_status batch_launch(gpunmf_batch *b, int iters) {
    GPUNMF_CUDA_TRY(cudaMemsetAsync(b->d_next, 0, sizeof(int), b->stream));
    batch_kernel<false><<<b->grid, kBatchThreads, batch_max_smem(), b->stream>>>(b->d_insts, b->d_order, b->count,
                                                                          b->d_next, b->V, b->W, b->H, b->eps,
                                                                          iters, BatchStop{0.f, nullptr});
    GPUNMF_CUDA_TRY(cudaGetLastError());
    return GPUNMF_OK;
}

extern "C" {

gpunmf_status gpunmf_batch_create(int count, const int *n, const int *m, const int *r, const float *const *V,
                                  const float *const *W, const float *const *H, float eps, gpunmf_batch **out) {
    if (!out || count <= 0 || !n || !m || !r || !V || !W || !H) {
        set_error("invalid batch arguments");
        return GPUNMF_ERR_INVALID;
    }
    *out = nullptr;
    int devs = 0;
    if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) {
        cudaGetLastError();
        set_error("no CUDA device available");
        return GPUNMF_ERR_NO_DEVICE;
    }
    gpunmf_batch *b = new (std::nothrow) gpunmf_batch();
    if (!b) return GPUNMF_ERR_NOMEM;
    b->count = count;
    b->eps = eps;
    b->h_insts.resize(count);
    for (int k = 0; k < count; k++) {
        if (n[k] <= 0 || m[k] <= 0 || r[k] <= 0 || rank_class(r[k]) == 0 || !V[k] || !W[k] || !H[k]) {
            set_error("instance %d: invalid shape or rank (batched ranks are 1..32)", k);
            delete b;
            return GPUNMF_ERR_INVALID;
        }
        BatchInst &d = b->h_insts[k];
        d.n = n[k]; d.m = m[k]; d.r = r[k]; d.cfg = default_cfg(r[k]);
        d.v = b->v_total; d.w = b->w_total; d.h = b->h_total;
        b->v_total += ((long long)n[k] * m[k] + 3) / 4 * 4;
        b->w_total += ((long long)n[k] * r[k] + 3) / 4 * 4;
        b->h_total += ((long long)r[k] * m[k] + 3) / 4 * 4;
    }
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_insts, sizeof(BatchInst) * count);
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_order, sizeof(int) * count);
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_next, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_res, sizeof(double) * count);
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->V, sizeof(float) * b->v_total);
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->W, sizeof(float) * b->w_total);
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->H, sizeof(float) * b->h_total);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(batch_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)batch_max_smem());
    if (e != cudaSuccess) {
        set_error("batch allocation failed: %s", cudaGetErrorString(e));
        cudaGetLastError();
        batch_free(b);
        return GPUNMF_ERR_NOMEM;
    }
    // stage through one pinned buffer per matrix kind, one copy each
    for (int kind = 0; kind < 3; kind++) {
        long long total = kind == 0 ? b->v_total : kind == 1 ? b->w_total : b->h_total;
        float *stage = nullptr;
        if (cudaHostAlloc((void **)&stage, sizeof(float) * total, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            set_error("pinned staging allocation failed");
            batch_free(b);
            return GPUNMF_ERR_NOMEM;
        }
        for (int k = 0; k < count; k++) {
            const BatchInst &d = b->h_insts[k];
            const float *src = kind == 0 ? V[k] : kind == 1 ? W[k] : H[k];
            long long off = kind == 0 ? d.v : kind == 1 ? d.w : d.h;
            long long cnt = kind == 0 ? (long long)d.n * d.m : kind == 1 ? (long long)d.n * d.r : (long long)d.r * d.m;
            std::copy(src, src + cnt, stage + off);
        }
        float *dst = kind == 0 ? b->V : kind == 1 ? b->W : b->H;
        cudaError_t ce = cudaMemcpyAsync(dst, stage, sizeof(float) * total, cudaMemcpyHostToDevice, b->stream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(b->stream);
        cudaFreeHost(stage);
        if (ce != cudaSuccess) {
            set_error("batch upload failed: %s", cudaGetErrorString(ce));
            batch_free(b);
            return GPUNMF_ERR_CUDA;
        }
    }
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel<false>, kBatchThreads, batch_max_smem());
    b->grid = std::max(1, sms * std::max(1, per_sm));
    gpunmf_status st = batch_upload_order(b);
    if (st != GPUNMF_OK) {
        batch_free(b);
        return st;
    }
    *out = b;
    return GPUNMF_OK;
}

gpunmf_status gpunmf_batch_destroy(gpunmf_batch *b) {
    if (!b) return GPUNMF_ERR_INVALID;
    cudaStreamSynchronize(b->stream);
    batch_free(b);
    return GPUNMF_OK;
}

// Run `iters` iterations of every instance: one persistent launch, captured in a CUDA graph
// (re-captured when iters changes) and replayed.  Returns without waiting.
gpunmf_status gpunmf_batch_run(gpunmf_batch *b, int iters) {
    if (!b || iters < 0) return GPUNMF_ERR_INVALID;
    if (iters == 0) return GPUNMF_OK;
    if (!b->graph || b->graph_iters != iters) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        cudaGraph_t g = nullptr;
        GPUNMF_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        gpunmf_status st = batch_launch(b, iters);
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (st != GPUNMF_OK || e != cudaSuccess) {
            // the capture may have produced a graph even when the launch or the capture failed
            if (g) cudaGraphDestroy(g);
            if (st != GPUNMF_OK) return st;
            GPUNMF_CUDA_TRY(e);
        }
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        GPUNMF_CUDA_TRY(e);
        b->graph_iters = iters;
    }
    GPUNMF_CUDA_TRY(cudaGraphLaunch(b->graph, b->stream));
    return GPUNMF_OK;
}

gpunmf_status gpunmf_batch_synchronize(gpunmf_batch *b) {
    if (!b) return GPUNMF_ERR_INVALID;
    GPUNMF_CUDA_TRY(cudaStreamSynchronize(b->stream));
    return GPUNMF_OK;
}

// Device time of `iters` iterations of the whole batch (one graph launch), in ms.
gpunmf_status gpunmf_batch_time(gpunmf_batch *b, int iters, float *ms) {
    if (!b || !ms) return GPUNMF_ERR_INVALID;
    cudaEvent_t e0, e1;
    GPUNMF_CUDA_TRY(cudaEventCreate(&e0));
    GPUNMF_CUDA_TRY(cudaEventCreate(&e1));
    gpunmf_status st = gpunmf_batch_run(b, iters);  // captures outside the timed region if needed
    if (st == GPUNMF_OK) {
        cudaStreamSynchronize(b->stream);
        cudaEventRecord(e0, b->stream);
        st = gpunmf_batch_run(b, iters);
        cudaEventRecord(e1, b->stream);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(ms, e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return st;
}

gpunmf_status gpunmf_batch_get(gpunmf_batch *b, int k, float *W, float *H) {
    if (!b || k < 0 || k >= b->count) return GPUNMF_ERR_INVALID;
    const BatchInst &d = b->h_insts[k];
    if (W) GPUNMF_CUDA_TRY(cudaMemcpyAsync(W, b->W + d.w, sizeof(float) * (size_t)d.n * d.r, cudaMemcpyDeviceToHost, b->stream));
    if (H) GPUNMF_CUDA_TRY(cudaMemcpyAsync(H, b->H + d.h, sizeof(float) * (size_t)d.r * d.m, cudaMemcpyDeviceToHost, b->stream));
    GPUNMF_CUDA_TRY(cudaStreamSynchronize(b->stream));
    return GPUNMF_OK;
}

// Relative residual of every instance (FP64 accumulation on the GPU).
gpunmf_status gpunmf_batch_residuals(gpunmf_batch *b, double *out) {
    if (!b || !out) return GPUNMF_ERR_INVALID;
    batch_residual_kernel<<<b->count, 256, 0, b->stream>>>(b->d_insts, b->count, b->V, b->W, b->H, b->d_res);
    GPUNMF_CUDA_TRY(cudaGetLastError());
    GPUNMF_CUDA_TRY(cudaMemcpyAsync(out, b->d_res, sizeof(double) * b->count, cudaMemcpyDeviceToHost, b->stream));
    GPUNMF_CUDA_TRY(cudaStreamSynchronize(b->stream));
    return GPUNMF_OK;
}

// Tile configuration of instance k (see gpunmf_batch_configs); the rank class must match.
gpunmf_status gpunmf_batch_set_config(gpunmf_batch *b, int k, int cfg) {
    if (!b || k < 0 || k >= b->count || cfg < 0 || cfg >= kBatchConfigs) return GPUNMF_ERR_INVALID;
    if (batch_cfg_rank(cfg) != rank_class(b->h_insts[k].r)) {
        set_error("config %d is for rank class %d, instance %d has r=%d", cfg, batch_cfg_rank(cfg), k,
                  b->h_insts[k].r);
        return GPUNMF_ERR_INVALID;
    }
    b->h_insts[k].cfg = cfg;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return GPUNMF_OK;
}

// Commit configuration changes (uploads descriptors and the largest-first order).
gpunmf_status gpunmf_batch_commit(gpunmf_batch *b) {
    if (!b) return GPUNMF_ERR_INVALID;
    return batch_upload_order(b);
}

// Number of tile configurations and the rank class of each (ranks[c], c < count).
int gpunmf_batch_configs(int *ranks, int cap) {
    for (int c = 0; c < kBatchConfigs && c < cap; c++)
        if (ranks) ranks[c] = batch_cfg_rank(c);
    return kBatchConfigs;
}

// Reset every instance's W and H to the given host values (same packing as create).
gpunmf_status gpunmf_batch_reset_factors(gpunmf_batch *b, const float *const *W, const float *const *H) {
    if (!b || !W || !H) return GPUNMF_ERR_INVALID;
    for (int k = 0; k < b->count; k++) {
        const BatchInst &d = b->h_insts[k];
        GPUNMF_CUDA_TRY(cudaMemcpyAsync(b->W + d.w, W[k], sizeof(float) * (size_t)d.n * d.r, cudaMemcpyHostToDevice, b->stream));
        GPUNMF_CUDA_TRY(cudaMemcpyAsync(b->H + d.h, H[k], sizeof(float) * (size_t)d.r * d.m, cudaMemcpyHostToDevice, b->stream));
    }
    GPUNMF_CUDA_TRY(cudaStreamSynchronize(b->stream));
    return GPUNMF_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Grouped training (src/examples/FacesNMF/FacesNMFDlg.cpp:582-656, TrainUsingGroups).
//
// V's first blocks*group columns are cut into `blocks` = floor(m/group) blocks of `group`
// consecutive columns; block s is an independent NMF of rank rs = floor(r/blocks).  Column
// blocks of a column-major matrix are contiguous, so the blocks of V and W need no packing; the
// diagonal blocks of H are gathered into a packed array and scattered back (zeros elsewhere in
// the block's columns, as :640-651 writes).  Two ways to run the blocks:
//   - multiplicative Euclidean, FP32, rs <= 32: every block is one instance of the persistent
//     batch kernel above, which samples the quality itself and stops the instance on the
//     reference's test (one launch for all blocks);
//   - any other rule or precision: one engine job per block (the same code as the class API),
//     up to 64 in flight on their own streams, driven round-robin by this thread; each job's
//     quality read-back is one iteration behind, so the host rarely waits.
// ---------------------------------------------------------------------------
namespace gpunmf {

__global__ void gather_h_blocks(const float *__restrict__ H, int r, int group, int rs, int blocks,
                                float *__restrict__ Hp) {
    const long long total = (long long)blocks * rs * group;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const long long s = k / ((long long)rs * group), rem = k % ((long long)rs * group);
        const long long u = rem / rs, a = rem % rs;  // packed block: rs x group column-major
        Hp[k] = H[(s * group + u) * r + s * rs + a];
    }
}

__global__ void scatter_h_blocks(float *__restrict__ H, int r, int group, int rs, int blocks,
                                 const float *__restrict__ Hp) {
    const long long total = (long long)blocks * group * r;  // the first blocks*group columns of H
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const long long col = k / r, row = k % r;
        const long long s = col / group, u = col % group, a = row - s * rs;
        H[k] = (a >= 0 && a < rs) ? Hp[s * rs * group + u * rs + a] : 0.f;
    }
}

static int ew_grid(long long count) {
    long long b = (count + 255) / 256;
    return (int)std::max(1LL, std::min(b, 8LL * kNumSMsGB300));
}

// one engine job per block, round-robin
static gpunmf_status grouped_jobs(int rule, int n, int group, int rs, int blocks, const float *dV, float *dW,
                                  float *dHp, float tol, int max_iters, float eps, int precision, int *iters_out) {
    struct Slot {
        gpunmf_job *j = nullptr;
        int s = -1, its = 0;
        float prev = 1.f;
    };
    const int window = std::min(blocks, 64);
    std::vector<Slot> slots(window);
    int next = 0, remaining = blocks;
    gpunmf_status st = GPUNMF_OK;
    const size_t vb = (size_t)n * group, wb = (size_t)n * rs, hb = (size_t)rs * group;
    auto start = [&](Slot &sl) -> gpunmf_status {
        sl.s = next++;
        sl.its = 0;
        gpunmf_status s2 = job_create_empty(rule, n, group, rs, eps, precision, nullptr, nullptr, false, &sl.j);
        if (s2 != GPUNMF_OK) return s2;
        cudaStream_t js = sl.j->stream;
        GPUNMF_CUDA_TRY(cudaMemcpyAsync(sl.j->V, dV + sl.s * vb, vb * sizeof(float), cudaMemcpyDeviceToDevice, js));
        GPUNMF_CUDA_TRY(cudaMemcpyAsync(sl.j->W, dW + sl.s * wb, wb * sizeof(float), cudaMemcpyDeviceToDevice, js));
        GPUNMF_CUDA_TRY(cudaMemcpyAsync(sl.j->H, dHp + sl.s * hb, hb * sizeof(float), cudaMemcpyDeviceToDevice, js));
        s2 = job_prepare(sl.j);
        sl.prev = sl.j->q_delta;  // QualityImprovement() of a new object (FacesNMFDlg.cpp:605)
        return s2;
    };
    auto finish = [&](Slot &sl) -> gpunmf_status {
        cudaStream_t js = sl.j->stream;
        GPUNMF_CUDA_TRY(cudaMemcpyAsync(dW + sl.s * wb, sl.j->W, wb * sizeof(float), cudaMemcpyDeviceToDevice, js));
        GPUNMF_CUDA_TRY(cudaMemcpyAsync(dHp + sl.s * hb, sl.j->H, hb * sizeof(float), cudaMemcpyDeviceToDevice, js));
        GPUNMF_CUDA_TRY(cudaStreamSynchronize(js));
        iters_out[sl.s] = sl.its;
        job_release(sl.j);
        sl.j = nullptr;
        remaining--;
        return GPUNMF_OK;
    };
    while (st == GPUNMF_OK && remaining > 0) {
        for (Slot &sl : slots) {
            if (!sl.j) {
                if (next >= blocks) continue;
                st = start(sl);
                if (st != GPUNMF_OK) break;
            }
            st = job_run(sl.j, 1, true);  // DoIteration(true) (FacesNMFDlg.cpp:610)
            if (st != GPUNMF_OK) break;
            sl.its++;
            bool done = sl.its >= max_iters;
            const float q = sl.j->q_delta;  // QualityImprovement() (:612-616)
            if (q != sl.prev) {
                if (q < tol) done = true;
                else sl.prev = q;
            }
            if (done) {
                st = finish(sl);
                if (st != GPUNMF_OK) break;
            }
        }
    }
    for (Slot &sl : slots)
        if (sl.j) job_release(sl.j);
    return st;
}

}  // namespace gpunmf

extern "C" gpunmf_status gpunmf_grouped_train(int rule, int n, int m, int r, int group, const float *V, float *W,
                                              float *H, float tol, int max_iters, float eps, int precision,
                                              int *iterations) {
    if (!V || !W || !H || n <= 0 || m <= 0 || r <= 0 || group <= 0 || max_iters <= 0 || !rule_valid(rule) ||
        !(eps >= 0.f) || (precision != GPUNMF_FP32 && precision != GPUNMF_BF16)) {
        set_error("invalid grouped-training arguments");
        return GPUNMF_ERR_INVALID;
    }
    const int blocks = m / group;
    const int rs = blocks > 0 ? r / blocks : 0;
    if (blocks < 1 || rs < 1) {
        set_error("grouped training needs group <= m and r >= m/group (group %d, m %d, r %d)", group, m, r);
        return GPUNMF_ERR_INVALID;
    }
    int devs = 0;
    if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) {
        cudaGetLastError();
        set_error("no CUDA device available");
        return GPUNMF_ERR_NO_DEVICE;
    }
    const bool batched = rule == GPUNMF_EUCLIDEAN && precision == GPUNMF_FP32 && rank_class(rs) != 0;
    const size_t vcount = (size_t)n * blocks * group, wcount = (size_t)n * blocks * rs, hcount = (size_t)r * m;
    const size_t hpcount = (size_t)blocks * rs * group;
    cudaStream_t s = nullptr;
    float *dV = nullptr, *dW = nullptr, *dH = nullptr, *dHp = nullptr;
    int *d_iters = nullptr, *d_order = nullptr, *d_next = nullptr;
    BatchInst *d_insts = nullptr;
    std::vector<int> h_iters(blocks, 0);
    gpunmf_status st = GPUNMF_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void **)&dV, vcount * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&dW, wcount * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&dH, hcount * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&dHp, hpcount * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_iters, blocks * sizeof(int));
    if (e != cudaSuccess) {
        set_error("grouped training allocation failed: %s", cudaGetErrorString(e));
        cudaGetLastError();
        st = GPUNMF_ERR_NOMEM;
    }
    // the blocks' V and W columns and the whole H (the columns outside the blocks come back as they were)
    if (st == GPUNMF_OK) {
        e = cudaMemcpyAsync(dV, V, vcount * sizeof(float), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dW, W, wcount * sizeof(float), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dH, H, hcount * sizeof(float), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) {
            gather_h_blocks<<<ew_grid(hpcount), 256, 0, s>>>(dH, r, group, rs, blocks, dHp);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("grouped training upload failed: %s", cudaGetErrorString(e));
            st = GPUNMF_ERR_CUDA;
        }
    }
    if (st == GPUNMF_OK && batched) {
        std::vector<BatchInst> insts(blocks);
        std::vector<int> order(blocks);
        for (int b = 0; b < blocks; b++) {
            BatchInst &d = insts[b];
            d.n = n; d.m = group; d.r = rs; d.cfg = default_cfg(rs);
            d.v = (long long)b * n * group;
            d.w = (long long)b * n * rs;
            d.h = (long long)b * rs * group;
            order[b] = b;
        }
        e = cudaMalloc((void **)&d_insts, blocks * sizeof(BatchInst));
        if (e == cudaSuccess) e = cudaMalloc((void **)&d_order, blocks * sizeof(int));
        if (e == cudaSuccess) e = cudaMalloc((void **)&d_next, sizeof(int));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_insts, insts.data(), blocks * sizeof(BatchInst), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_order, order.data(), blocks * sizeof(int), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(d_next, 0, sizeof(int), s);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(batch_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)batch_max_smem());
        int dev = 0, sms = 0, per_sm = 0;
        if (e == cudaSuccess) e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel<true>, kBatchThreads,
                                                              batch_max_smem());
        if (e == cudaSuccess) {
            const int grid = std::max(1, std::min(blocks, sms * std::max(1, per_sm)));
            batch_kernel<true><<<grid, kBatchThreads, batch_max_smem(), s>>>(d_insts, d_order, blocks, d_next, dV, dW,
                                                                             dHp, eps, max_iters,
                                                                             BatchStop{tol, d_iters});
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h_iters.data(), d_iters, blocks * sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) {
            set_error("grouped batch launch failed: %s", cudaGetErrorString(e));
            cudaGetLastError();
            st = GPUNMF_ERR_CUDA;
        }
    } else if (st == GPUNMF_OK) {
        st = grouped_jobs(rule, n, group, rs, blocks, dV, dW, dHp, tol, max_iters, eps, precision, h_iters.data());
    }
    if (st == GPUNMF_OK) {
        scatter_h_blocks<<<ew_grid((long long)blocks * group * r), 256, 0, s>>>(dH, r, group, rs, blocks, dHp);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(W, dW, wcount * sizeof(float), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(H, dH, hcount * sizeof(float), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("grouped training read-back failed: %s", cudaGetErrorString(e));
            st = GPUNMF_ERR_CUDA;
        } else if (iterations) {
            std::copy(h_iters.begin(), h_iters.end(), iterations);
        }
    }
    if (s) cudaStreamSynchronize(s);
    void *ptrs[] = {dV, dW, dH, dHp, d_iters, d_order, d_next, d_insts};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (s) cudaStreamDestroy(s);
    return st;
}
