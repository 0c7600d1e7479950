// FP32 CUDA-core kernels of the plain (drop-in) NMF path.
//
// The reference runs its factor products through cuBLAS SGEMM
// (src/memory/DeviceMatrix.h:195-227) and its updates through the kernels of
// src/cuda/nmf/nmf_kernels.cu.  Here one register-tiled SGEMM template covers
// every product shape of all four rules: operands are read through small
// "loader" functors (plain column-major, transposed view, or the KL ratio
// V/(WH+eps), or V/(WH+eps) - 1 for the additive KL rule, formed on the fly),
// and the epilogue either stores, stores split-K partial products, applies a
// KL update in place, or reduces a function of (V, WH)
// into per-CTA FP64 partials (quality / residual) without storing WH.
#include <math.h>

#include "common.cuh"
#include "kernels.h"

namespace gpunmf {

// ------------------------------------------------------------------------
// operand loaders: element (row, col) of an operand; kRowContig says that
// consecutive rows are adjacent in memory (an untransposed column-major view)
// ------------------------------------------------------------------------
struct LdCM {
    const float *p;
    long long ld;
    static constexpr bool kRowContig = true;
    __device__ __forceinline__ float operator()(int row, int col) const {
        return __ldg(p + (long long)col * ld + row);
    }
};
struct LdCMT {  // transpose view: op(row, col) = X(col, row)
    const float *p;
    long long ld;
    static constexpr bool kRowContig = false;
    __device__ __forceinline__ float operator()(int row, int col) const {
        return __ldg(p + (long long)row * ld + col);
    }
};
struct LdRatio {  // V(row,col) / (WH(row,col) + eps), both column-major with ld
    const float *V, *WH;
    long long ld;
    float eps;
    static constexpr bool kRowContig = true;
    __device__ __forceinline__ float operator()(int row, int col) const {
        long long o = (long long)col * ld + row;
        return __ldg(V + o) / (__ldg(WH + o) + eps);
    }
};

struct LdRatioM1 {  // V/(WH+eps) - 1: the additive KL gradient term (nmf_kernels_additive_divergence.cu:90,159)
    const float *V, *WH;
    long long ld;
    float eps;
    static constexpr bool kRowContig = true;
    __device__ __forceinline__ float operator()(int row, int col) const {
        long long o = (long long)col * ld + row;
        return __ldg(V + o) / (__ldg(WH + o) + eps) - 1.0f;
    }
};

// ------------------------------------------------------------------------
// epilogues
// ------------------------------------------------------------------------
struct EpiStore {  // C[z*zstride + j*ldc + i] = c
    float *C;
    long long ldc, zstride;
    static constexpr bool kReduce = false;
    __device__ __forceinline__ void operator()(int i, int j, float c, int z) const {
        C[(long long)z * zstride + (long long)j * ldc + i] = c;
    }
};
struct EpiKLUpdate {  // X(i,j) *= c / sums[by_row ? i : j]   (nmf_kernels.cu:289,337)
    float *X;
    long long ldx;
    const float *sums;
    bool by_row;
    static constexpr bool kReduce = false;
    __device__ __forceinline__ void operator()(int i, int j, float c, int) const {
        float *x = X + (long long)j * ldx + i;
        *x *= (c / sums[by_row ? i : j]);
    }
};
struct EpiAKLUpdate {  // X(i,j) = max(0, x + (x / sums[..]) * c)  (nmf_kernels_additive_divergence.cu:101-104)
    float *X;
    long long ldx;
    const float *sums;
    bool by_row;
    static constexpr bool kReduce = false;
    __device__ __forceinline__ void operator()(int i, int j, float c, int) const {
        float *x = X + (long long)j * ldx + i;
        float v = *x + (*x / sums[by_row ? i : j]) * c;
        *x = v < 0.0f ? 0.0f : v;
    }
};
struct EpiQuality {  // sum V*log10(WH+eps) - WH   (nmf_kernels_quality.cu:35)
    const float *V;
    long long ldv;
    float eps;
    double *partial;
    static constexpr bool kReduce = true;
    static constexpr int kTerms = 1;
    __device__ __forceinline__ void term(int i, int j, float wh, double *t) const {
        float v = __ldg(V + (long long)j * ldv + i);
        t[0] += (double)(v * log10f(wh + eps) - wh);
    }
};
struct EpiResidual {  // sum (V-WH)^2 and sum V^2
    const float *V;
    long long ldv;
    double *partial;
    static constexpr bool kReduce = true;
    static constexpr int kTerms = 2;
    __device__ __forceinline__ void term(int i, int j, float wh, double *t) const {
        float v = __ldg(V + (long long)j * ldv + i);
        double d = (double)v - (double)wh;
        t[0] += d * d;
        t[1] += (double)v * (double)v;
    }
};

// ------------------------------------------------------------------------
// register-tiled SGEMM: C (M x N) = op(A) (M x K) * op(B) (K x N), over
// k in [blockIdx.z*kchunk, min(K, (blockIdx.z+1)*kchunk)).  Two shared
// buffers, the next tile is fetched into registers while the current one
// is multiplied.
// ------------------------------------------------------------------------
template <int BM, int BN, int BK, int TM, int TN, class LA, class LB, class Epi>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    gemm_f32_kernel(int M, int N, int K, int kchunk, LA la, LB lb, Epi epi) {
    constexpr int NT = (BM / TM) * (BN / TN);
    constexpr int TXM = BM / TM;  // threads along M
    constexpr int PAD = 4;
    constexpr int AL = BM * BK / NT, BL = BK * BN / NT;
    static_assert((BM * BK) % NT == 0 && (BK * BN) % NT == 0, "tile/threads mismatch");
    static_assert(TM % 4 == 0 && TN % 4 == 0, "vector width");
    __shared__ __align__(16) float As[2][BK][BM + PAD];
    __shared__ __align__(16) float Bs[2][BK][BN + PAD];

    const int tid = threadIdx.x;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int kb = blockIdx.z * kchunk;
    const int ke = min(K, kb + kchunk);
    float ra[AL], rb[BL];

    auto a_index = [](int idx, int &i, int &k) {
        if (LA::kRowContig) { i = idx % BM; k = idx / BM; }
        else                { k = idx % BK; i = idx / BK; }
    };
    auto b_index = [](int idx, int &k, int &j) {
        if (LB::kRowContig) { k = idx % BK; j = idx / BK; }
        else                { j = idx % BN; k = idx / BN; }
    };
    auto gload = [&](int k0) {
#pragma unroll
        for (int e = 0; e < AL; e++) {
            int i, k;
            a_index(tid + e * NT, i, k);
            int gi = m0 + i, gk = k0 + k;
            ra[e] = (gi < M && gk < ke) ? la(gi, gk) : 0.f;
        }
#pragma unroll
        for (int e = 0; e < BL; e++) {
            int k, j;
            b_index(tid + e * NT, k, j);
            int gk = k0 + k, gj = n0 + j;
            rb[e] = (gk < ke && gj < N) ? lb(gk, gj) : 0.f;
        }
    };
    auto sstore = [&](int buf) {
#pragma unroll
        for (int e = 0; e < AL; e++) {
            int i, k;
            a_index(tid + e * NT, i, k);
            As[buf][k][i] = ra[e];
        }
#pragma unroll
        for (int e = 0; e < BL; e++) {
            int k, j;
            b_index(tid + e * NT, k, j);
            Bs[buf][k][j] = rb[e];
        }
    };

    float acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) acc[i][j] = 0.f;

    const int tmi = tid % TXM, tni = tid / TXM;
    if (kb < ke) {
        gload(kb);
        sstore(0);
    }
    __syncthreads();
    int buf = 0;
    for (int k0 = kb; k0 < ke; k0 += BK) {
        const bool more = k0 + BK < ke;
        if (more) gload(k0 + BK);
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            float a[TM], b[TN];
#pragma unroll
            for (int q = 0; q < TM; q += 4)
                *reinterpret_cast<float4 *>(&a[q]) =
                    *reinterpret_cast<const float4 *>(&As[buf][kk][tmi * TM + q]);
#pragma unroll
            for (int q = 0; q < TN; q += 4)
                *reinterpret_cast<float4 *>(&b[q]) =
                    *reinterpret_cast<const float4 *>(&Bs[buf][kk][tni * TN + q]);
#pragma unroll
            for (int i = 0; i < TM; i++)
#pragma unroll
                for (int j = 0; j < TN; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        if (more) sstore(buf ^ 1);
        __syncthreads();
        buf ^= 1;
    }

    if constexpr (Epi::kReduce) {
        __shared__ double red[32];
        double t[Epi::kTerms];
#pragma unroll
        for (int q = 0; q < Epi::kTerms; q++) t[q] = 0.0;
#pragma unroll
        for (int ii = 0; ii < TM; ii++)
#pragma unroll
            for (int jj = 0; jj < TN; jj++) {
                int i = m0 + tmi * TM + ii, j = n0 + tni * TN + jj;
                if (i < M && j < N) epi.term(i, j, acc[ii][jj], t);
            }
        const long long cta = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
#pragma unroll
        for (int q = 0; q < Epi::kTerms; q++) {
            double s = block_sum(t[q], red);
            if (tid == 0) epi.partial[cta * Epi::kTerms + q] = s;
        }
    } else {
#pragma unroll
        for (int jj = 0; jj < TN; jj++)
#pragma unroll
            for (int ii = 0; ii < TM; ii++) {
                int i = m0 + tmi * TM + ii, j = n0 + tni * TN + jj;
                if (i < M && j < N) epi(i, j, acc[ii][jj], blockIdx.z);
            }
    }
}

// ------------------------------------------------------------------------
// tile selection
// ------------------------------------------------------------------------
enum TileKind { kSquare, kSkinnyM64, kSkinnyM32, kSkinnyN64, kSkinnyN32, kSmall };
struct TileDims { int bm, bn, bk; };

static TileKind pick_tile(int M, int N) {
    if (M <= 32 && N > 64) return kSkinnyM32;
    if (M <= 64 && N > 64) return kSkinnyM64;
    if (N <= 32 && M > 64) return kSkinnyN32;
    if (N <= 64 && M > 64) return kSkinnyN64;
    if (M <= 64 && N <= 64) return kSmall;
    return kSquare;
}
static TileDims tile_dims(TileKind t) {
    switch (t) {
        case kSkinnyM32: return {32, 128, 16};
        case kSkinnyM64: return {64, 64, 16};   // 64 threads, 8 x 8 per thread
        case kSkinnyN32: return {128, 32, 16};
        case kSkinnyN64: return {64, 64, 16};
        case kSmall: return {64, 64, 16};
        default: return {128, 128, 8};
    }
}

// Split-K count.  The long-K products (W'V, VH', their KL forms) have few output tiles, so K is
// split; what bounds them is the busiest SM: (CTAs on it) x (K per slice).  The count that
// minimises that, with at least four CTAs per SM counted (fewer do not keep an SM busy), is
// taken, the smallest among those within 1% of the least.  At 8192 x 8192, r = 64 this is 19
// slices (2432 CTAs of 64 x 64, 16 per SM): 233 us for W'V against 311 us with 5 slices.
static int splits_for(int M, int N, int K, TileDims d) {
    const long long tiles = (long long)ceil_div(M, d.bm) * ceil_div(N, d.bn);
    if (tiles >= 4LL * kNumSMsGB300) return 1;
    int maxs = K / 64;  // keep at least 64 of K per slice
    if (maxs < 1) return 1;
    if (maxs > 64) maxs = 64;
    auto cost = [&](int s) {
        long long kc = (long long)ceil_div(ceil_div(K, s), d.bk) * d.bk;
        long long ctas = tiles * ceil_div(K, kc);
        long long per_sm = (ctas + kNumSMsGB300 - 1) / kNumSMsGB300;
        if (per_sm < 4) per_sm = 4;
        return per_sm * kc;
    };
    long long least = cost(1);
    for (int s = 2; s <= maxs; s++) least = cost(s) < least ? cost(s) : least;
    for (int s = 1; s <= maxs; s++)
        if (cost(s) * 100 <= least * 101) return s;
    return 1;
}

int gemm_f32_splits(int M, int N, int K) { return splits_for(M, N, K, tile_dims(pick_tile(M, N))); }

template <class LA, class LB, class Epi>
static cudaError_t launch_tiled(TileKind t, int M, int N, int K, int splits, LA la, LB lb, Epi epi,
                                cudaStream_t s) {
    TileDims d = tile_dims(t);
    int kchunk = ceil_div(K, splits);
    kchunk = ceil_div(kchunk, d.bk) * d.bk;
    if (kchunk <= 0) kchunk = d.bk;
    dim3 grid(ceil_div(M, d.bm), ceil_div(N, d.bn), splits);
    switch (t) {
        case kSkinnyM32: gemm_f32_kernel<32, 128, 16, 4, 4, LA, LB, Epi><<<grid, 256, 0, s>>>(M, N, K, kchunk, la, lb, epi); break;
        case kSkinnyM64:
        case kSkinnyN64: gemm_f32_kernel<64, 64, 16, 8, 8, LA, LB, Epi><<<grid, 64, 0, s>>>(M, N, K, kchunk, la, lb, epi); break;
        case kSkinnyN32: gemm_f32_kernel<128, 32, 16, 4, 4, LA, LB, Epi><<<grid, 256, 0, s>>>(M, N, K, kchunk, la, lb, epi); break;
        case kSmall: gemm_f32_kernel<64, 64, 16, 4, 4, LA, LB, Epi><<<grid, 256, 0, s>>>(M, N, K, kchunk, la, lb, epi); break;
        default: gemm_f32_kernel<128, 128, 8, 8, 8, LA, LB, Epi><<<grid, 256, 0, s>>>(M, N, K, kchunk, la, lb, epi); break;
    }
    return cudaGetLastError();
}

template <class LA, class LB>
static cudaError_t gemm_store(int M, int N, int K, LA la, LB lb, float *C, long long ldc, int splits,
                              cudaStream_t s) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    TileKind t = pick_tile(M, N);
    // short K (the Gram-times-factor products, K = r): the same 64 x 64 tiles with 4 x 4 outputs per
    // thread, four times the warps to hide the loads
    if (K <= 128 && (t == kSkinnyM64 || t == kSkinnyN64)) t = kSmall;
    if (splits < 1) splits = 1;
    EpiStore e{C, splits == 1 ? ldc : (long long)M, splits == 1 ? 0LL : (long long)M * N};
    return launch_tiled(t, M, N, K, splits, la, lb, e, s);
}

cudaError_t gemm_f32(int M, int N, int K, F32Operand A, F32Operand B, float *C, long long ldc,
                     int splits, cudaStream_t s) {
    if (!A.t && !B.t) return gemm_store(M, N, K, LdCM{A.p, A.ld}, LdCM{B.p, B.ld}, C, ldc, splits, s);
    if (A.t && !B.t) return gemm_store(M, N, K, LdCMT{A.p, A.ld}, LdCM{B.p, B.ld}, C, ldc, splits, s);
    if (!A.t && B.t) return gemm_store(M, N, K, LdCM{A.p, A.ld}, LdCMT{B.p, B.ld}, C, ldc, splits, s);
    return gemm_store(M, N, K, LdCMT{A.p, A.ld}, LdCMT{B.p, B.ld}, C, ldc, splits, s);
}

template <class LR>
static cudaError_t ratio_left(int M, int N, int K, LR ra, F32Operand B, float *P, int splits, cudaStream_t s) {
    if (B.t) return gemm_store(M, N, K, ra, LdCMT{B.p, B.ld}, P, M, splits, s);
    return gemm_store(M, N, K, ra, LdCM{B.p, B.ld}, P, M, splits, s);
}

template <class LR>
static cudaError_t ratio_right(int M, int N, int K, F32Operand A, LR rb, float *P, int splits, cudaStream_t s) {
    if (A.t) return gemm_store(M, N, K, LdCMT{A.p, A.ld}, rb, P, M, splits, s);
    return gemm_store(M, N, K, LdCM{A.p, A.ld}, rb, P, M, splits, s);
}

cudaError_t gemm_f32_ratio_left(int M, int N, int K, const float *V, const float *WH, long long ldv,
                                float eps, F32Operand B, float *P, int splits, cudaStream_t s, bool minus_one) {
    if (minus_one) return ratio_left(M, N, K, LdRatioM1{V, WH, ldv, eps}, B, P, splits, s);
    return ratio_left(M, N, K, LdRatio{V, WH, ldv, eps}, B, P, splits, s);
}

cudaError_t gemm_f32_ratio_right(int M, int N, int K, F32Operand A, const float *V, const float *WH,
                                 long long ldv, float eps, float *P, int splits, cudaStream_t s, bool minus_one) {
    if (minus_one) return ratio_right(M, N, K, A, LdRatioM1{V, WH, ldv, eps}, P, splits, s);
    return ratio_right(M, N, K, A, LdRatio{V, WH, ldv, eps}, P, splits, s);
}

int wh_reduce_ctas(int n, int m) {
    TileDims d = tile_dims(pick_tile(n, m));
    return ceil_div(n, d.bm) * ceil_div(m, d.bn);
}

cudaError_t wh_quality_f32(int n, int m, int r, const float *W, const float *H, const float *V,
                           float eps, double *partial, cudaStream_t s) {
    EpiQuality e{V, (long long)n, eps, partial};
    return launch_tiled(pick_tile(n, m), n, m, r, 1, LdCM{W, n}, LdCM{H, r}, e, s);
}

cudaError_t wh_residual_f32(int n, int m, int r, const float *W, const float *H, const float *V,
                            double *partial, cudaStream_t s) {
    EpiResidual e{V, (long long)n, partial};
    return launch_tiled(pick_tile(n, m), n, m, r, 1, LdCM{W, n}, LdCM{H, r}, e, s);
}

// ------------------------------------------------------------------------
// reference-shaped KL updates over a stored WH: one launch, in place
// ------------------------------------------------------------------------
cudaError_t kl_update_h_ref(float *H, const float *W, const float *V, const float *WH,
                            const float *sumW, int n, int m, int r, float eps, cudaStream_t s) {
    // acc(a,u) = sum_i W(i,a) * [V(i,u)/(WH(i,u)+eps)];  H(a,u) *= acc / sumW[a]
    EpiKLUpdate e{H, (long long)r, sumW, true};
    return launch_tiled(pick_tile(r, m), r, m, n, 1, LdCMT{W, n}, LdRatio{V, WH, n, eps}, e, s);
}

cudaError_t kl_update_w_ref(float *W, const float *H, const float *V, const float *WH,
                            const float *sumH, int n, int m, int r, float eps, cudaStream_t s) {
    // acc(i,a) = sum_u [V(i,u)/(WH(i,u)+eps)] * H(a,u);  W(i,a) *= acc / sumH[a]
    EpiKLUpdate e{W, (long long)n, sumH, false};
    return launch_tiled(pick_tile(n, r), n, r, m, 1, LdRatio{V, WH, n, eps}, LdCMT{H, r}, e, s);
}

cudaError_t akl_update_h_ref(float *H, const float *W, const float *V, const float *WH,
                             const float *sumW, int n, int m, int r, float eps, cudaStream_t s) {
    // acc(a,u) = sum_i W(i,a) * [V(i,u)/(WH(i,u)+eps) - 1];  H(a,u) = max(0, h + (h/sumW[a]) acc)
    EpiAKLUpdate e{H, (long long)r, sumW, true};
    return launch_tiled(pick_tile(r, m), r, m, n, 1, LdCMT{W, n}, LdRatioM1{V, WH, n, eps}, e, s);
}

cudaError_t akl_update_w_ref(float *W, const float *H, const float *V, const float *WH,
                             const float *sumH, int n, int m, int r, float eps, cudaStream_t s) {
    // acc(i,a) = sum_u [V(i,u)/(WH(i,u)+eps) - 1] * H(a,u);  W(i,a) = max(0, w + (w/sumH[a]) acc)
    EpiAKLUpdate e{W, (long long)n, sumH, false};
    return launch_tiled(pick_tile(n, r), n, r, m, 1, LdRatioM1{V, WH, n, eps}, LdCMT{H, r}, e, s);
}

// ------------------------------------------------------------------------
// elementwise and reduction kernels
// ------------------------------------------------------------------------
constexpr int kEwThreads = 256;

// sum_z P[z*count + k] in z order; eight independent loads in flight per step
__device__ __forceinline__ float sum_slices(const float *__restrict__ P, int splits, long long count, long long k) {
    float acc = P[k];
    int z = 1;
    for (; z + 8 <= splits; z += 8) {
        float v[8];
#pragma unroll
        for (int q = 0; q < 8; q++) v[q] = P[(long long)(z + q) * count + k];
#pragma unroll
        for (int q = 0; q < 8; q++) acc += v[q];
    }
    for (; z < splits; z++) acc += P[(long long)z * count + k];
    return acc;
}

__device__ __forceinline__ float4 sum_slices4(const float4 *__restrict__ P, int splits, long long count4,
                                              long long k) {
    float4 acc = P[k];
    int z = 1;
    for (; z + 4 <= splits; z += 4) {
        float4 v[4];
#pragma unroll
        for (int q = 0; q < 4; q++) v[q] = P[(long long)(z + q) * count4 + k];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            acc.x += v[q].x; acc.y += v[q].y; acc.z += v[q].z; acc.w += v[q].w;
        }
    }
    for (; z < splits; z++) {
        float4 q = P[(long long)z * count4 + k];
        acc.x += q.x; acc.y += q.y; acc.z += q.z; acc.w += q.w;
    }
    return acc;
}

static int ew_blocks(long long count, int per_thread = 4) {
    long long b = (count + (long long)kEwThreads * per_thread - 1) / ((long long)kEwThreads * per_thread);
    long long cap = 8LL * kNumSMsGB300;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

__global__ void euclid_update_kernel(float *__restrict__ X, const float *__restrict__ P, int splits,
                                     const float *__restrict__ D, long long count, float eps) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count; k += stride) {
        float num = sum_slices(P, splits, count, k);
        X[k] *= num / (D[k] + eps);
    }
}

__global__ void euclid_update_kernel_v4(float4 *__restrict__ X, const float4 *__restrict__ P, int splits,
                                        const float4 *__restrict__ D, long long count4, float eps) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count4; k += stride) {
        float4 num = sum_slices4(P, splits, count4, k);
        float4 d = D[k], x = X[k];
        x.x *= num.x / (d.x + eps);
        x.y *= num.y / (d.y + eps);
        x.z *= num.z / (d.z + eps);
        x.w *= num.w / (d.w + eps);
        X[k] = x;
    }
}

static bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }

cudaError_t euclid_update(float *X, const float *P, int splits, const float *D, long long count,
                          float eps, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    if ((count & 3) == 0 && aligned16(X) && aligned16(P) && aligned16(D)) {
        long long c4 = count >> 2;
        euclid_update_kernel_v4<<<ew_blocks(c4, 2), kEwThreads, 0, s>>>(
            reinterpret_cast<float4 *>(X), reinterpret_cast<const float4 *>(P), splits,
            reinterpret_cast<const float4 *>(D), c4, eps);
    } else {
        euclid_update_kernel<<<ew_blocks(count), kEwThreads, 0, s>>>(X, P, splits, D, count, eps);
    }
    return cudaGetLastError();
}

// X = max(0, X + (X / D) * (num - D))   (nmf_kernels.cu:31-38; no epsilon, as there)
__device__ __forceinline__ float additive_step(float x, float num, float d) {
    float v = x + (x / d) * (num - d);
    return v < 0.0f ? 0.0f : v;
}

__global__ void additive_update_kernel(float *__restrict__ X, const float *__restrict__ P, int splits,
                                       const float *__restrict__ D, long long count) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count; k += stride)
        X[k] = additive_step(X[k], sum_slices(P, splits, count, k), D[k]);
}

__global__ void additive_update_kernel_v4(float4 *__restrict__ X, const float4 *__restrict__ P, int splits,
                                          const float4 *__restrict__ D, long long count4) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count4; k += stride) {
        float4 num = sum_slices4(P, splits, count4, k);
        float4 d = D[k], x = X[k];
        x.x = additive_step(x.x, num.x, d.x);
        x.y = additive_step(x.y, num.y, d.y);
        x.z = additive_step(x.z, num.z, d.z);
        x.w = additive_step(x.w, num.w, d.w);
        X[k] = x;
    }
}

cudaError_t additive_update(float *X, const float *P, int splits, const float *D, long long count,
                            cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    if ((count & 3) == 0 && aligned16(X) && aligned16(P) && aligned16(D)) {
        long long c4 = count >> 2;
        additive_update_kernel_v4<<<ew_blocks(c4, 2), kEwThreads, 0, s>>>(
            reinterpret_cast<float4 *>(X), reinterpret_cast<const float4 *>(P), splits,
            reinterpret_cast<const float4 *>(D), c4);
    } else {
        additive_update_kernel<<<ew_blocks(count), kEwThreads, 0, s>>>(X, P, splits, D, count);
    }
    return cudaGetLastError();
}

__global__ void sum_partials_kernel(float *__restrict__ out, const float *__restrict__ P, int splits,
                                    long long count) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count; k += stride) {
        out[k] = sum_slices(P, splits, count, k);
    }
}

cudaError_t sum_partials(float *out, const float *P, int splits, long long count, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    sum_partials_kernel<<<ew_blocks(count), kEwThreads, 0, s>>>(out, P, splits, count);
    return cudaGetLastError();
}

__global__ void kl_update_kernel(float *__restrict__ X, const float *__restrict__ P, int splits,
                                 const float *__restrict__ sums, long long count, long long div,
                                 long long mod) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count; k += stride) {
        float acc = sum_slices(P, splits, count, k);
        X[k] *= (acc / sums[(k / div) % mod]);
    }
}

__global__ void akl_update_kernel(float *__restrict__ X, const float *__restrict__ P, int splits,
                                  const float *__restrict__ sums, long long count, long long div,
                                  long long mod) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count; k += stride) {
        float acc = sum_slices(P, splits, count, k);
        float x = X[k];
        float v = x + (x / sums[(k / div) % mod]) * acc;
        X[k] = v < 0.0f ? 0.0f : v;
    }
}

cudaError_t kl_update(float *X, const float *P, int splits, const float *sums, long long count,
                      long long div, long long mod, cudaStream_t s, bool additive) {
    if (count <= 0) return cudaSuccess;
    if (additive)
        akl_update_kernel<<<ew_blocks(count), kEwThreads, 0, s>>>(X, P, splits, sums, count, div, mod);
    else
        kl_update_kernel<<<ew_blocks(count), kEwThreads, 0, s>>>(X, P, splits, sums, count, div, mod);
    return cudaGetLastError();
}

// sums over contiguous columns: one block per column a of a column-major matrix (rows x cols)
__global__ void col_sums_kernel(const float *__restrict__ X, int rows, float eps, float *__restrict__ out) {
    __shared__ double red[32];
    const float *col = X + (long long)blockIdx.x * rows;
    float s = 0.f;
#pragma unroll 8
    for (int i = threadIdx.x; i < rows; i += blockDim.x) s += col[i];
    double t = block_sum((double)s, red);
    if (threadIdx.x == 0) {
        float v = (float)t;
        out[blockIdx.x] = v < eps ? eps : v;
    }
}

// sums over rows of a column-major r x m matrix: one block per row a (strided reads, as the
// reference's SumH; H is small and L2-resident)
__global__ void row_sums_kernel(const float *__restrict__ H, int r, int m, float eps, float *__restrict__ out) {
    __shared__ double red[32];
    const int a = blockIdx.x;
    float s = 0.f;
#pragma unroll 8
    for (int u = threadIdx.x; u < m; u += blockDim.x) s += H[(long long)u * r + a];
    double t = block_sum((double)s, red);
    if (threadIdx.x == 0) {
        float v = (float)t;
        out[a] = v < eps ? eps : v;
    }
}

cudaError_t col_sums(const float *W, int n, int r, float eps, float *sums, cudaStream_t s) {
    if (r <= 0) return cudaSuccess;
    col_sums_kernel<<<r, 256, 0, s>>>(W, n, eps, sums);
    return cudaGetLastError();
}

cudaError_t row_sums(const float *H, int r, int m, float eps, float *sums, cudaStream_t s) {
    if (r <= 0) return cudaSuccess;
    row_sums_kernel<<<r, 256, 0, s>>>(H, r, m, eps, sums);
    return cudaGetLastError();
}

int quality_ew_ctas(long long count) { return ew_blocks(count, 8); }

__global__ void quality_ew_kernel(const float *__restrict__ V, const float *__restrict__ WH, long long count,
                                  float eps, double *__restrict__ partial) {
    __shared__ double red[32];
    double t = 0.0;
    long long stride = (long long)gridDim.x * blockDim.x;
#pragma unroll 4
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count; k += stride) {
        float wh = WH[k];
        t += (double)(V[k] * log10f(wh + eps) - wh);
    }
    double s = block_sum(t, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

cudaError_t quality_ew(const float *V, const float *WH, long long count, float eps, double *partial,
                       cudaStream_t s) {
    quality_ew_kernel<<<quality_ew_ctas(count), kEwThreads, 0, s>>>(V, WH, count, eps, partial);
    return cudaGetLastError();
}

__global__ void kl_objective_kernel(const float *__restrict__ V, const float *__restrict__ WH, long long count,
                                    double *__restrict__ partial) {
    __shared__ double red[32];
    double t = 0.0;
    long long stride = (long long)gridDim.x * blockDim.x;
#pragma unroll 4
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count; k += stride) {
        double v = V[k], wh = WH[k];
        t += (v > 0.0 ? v * log(v / wh) : 0.0) - v + wh;
    }
    double s = block_sum(t, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

cudaError_t kl_objective_ew(const float *V, const float *WH, long long count, double *partial,
                            cudaStream_t s) {
    kl_objective_kernel<<<quality_ew_ctas(count), kEwThreads, 0, s>>>(V, WH, count, partial);
    return cudaGetLastError();
}

__global__ void finalize_kernel(const double *__restrict__ partial, int count, int terms, int mode,
                                float *out_f, double *out_d) {
    __shared__ double red[32];
    double s0 = 0.0, s1 = 0.0;
    for (int c = threadIdx.x; c < count; c += blockDim.x) {
        s0 += partial[(long long)c * terms];
        if (terms > 1) s1 += partial[(long long)c * terms + 1];
    }
    s0 = block_sum(s0, red);
    s1 = block_sum(s1, red);
    if (threadIdx.x == 0) {
        if (mode == 0) {
            if (out_f) out_f[0] = (float)s0;
            if (out_d) out_d[0] = s0;
        } else {
            double rr = s1 > 0.0 ? sqrt(s0 / s1) : 0.0;
            if (out_d) out_d[0] = rr;
            if (out_f) out_f[0] = (float)rr;
        }
    }
}

cudaError_t finalize_partials(const double *partial, int count, int terms, int mode, float *out_f,
                              double *out_d, cudaStream_t s) {
    finalize_kernel<<<1, 512, 0, s>>>(partial, count, terms, mode, out_f, out_d);
    return cudaGetLastError();
}

}  // namespace gpunmf
