// Batched multiplicative-update NMF: thousands of small, uneven Euclidean
// factorisations in one persistent launch.
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
#include "kernels.h"

namespace gpunmf {

struct BatchInst {
    long long v, w, h;  // offsets (floats) into the packed V, W, H buffers
    int n, m, r, cfg;
};

constexpr int kBatchThreads = 256;
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

    __device__ __noinline__ static void run(const BatchInst &d, const float *__restrict__ Vall, float *__restrict__ Wall,
                               float *__restrict__ Hall, float eps, int iters, float *sm) {
        const int n = d.n, m = d.m, r = d.r;
        const float *V = Vall + d.v;
        float *W = Wall + d.w;
        float *H = Hall + d.h;
        float *sG = sm + OFF_G, *sV = sm + OFF_V, *sF = sm + OFF_F, *sX = sm + OFF_X;
        const int tid = threadIdx.x;
        const int ag = tid % AG, ug = tid / AG;

        gram_init(sG, W, n, n, r, true, sF);  // G = W'W

        for (int it = 0; it < iters; it++) {
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
        }
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

__global__ void __launch_bounds__(kBatchThreads, 3)
    batch_kernel(const BatchInst *__restrict__ insts, const int *__restrict__ order, int count,
                 int *__restrict__ next, const float *__restrict__ V, float *__restrict__ W, float *__restrict__ H,
                 float eps, int iters) {
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
    case C: InstanceRunner<R, BC, BI>::run(d, V, W, H, eps, iters, bsm); break;
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
    batch_kernel<<<b->grid, kBatchThreads, batch_max_smem(), b->stream>>>(b->d_insts, b->d_order, b->count,
                                                                          b->d_next, b->V, b->W, b->H, b->eps,
                                                                          iters);
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
        e = cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)batch_max_smem());
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
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel, kBatchThreads, batch_max_smem());
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
        if (st != GPUNMF_OK) return st;
        GPUNMF_CUDA_TRY(e);
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
