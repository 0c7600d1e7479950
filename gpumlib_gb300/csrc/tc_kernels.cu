// BF16 tensor-core path (tcgen05 + TMA) of the Euclidean multiplicative update.
//
// Data layout in HBM (per job, beside the FP32 masters V, W, H):
//   Vb   n x m  BF16, column-major, ld = ceil8(n)   (V itself: rows i contiguous)
//   Vbt  m x n  BF16, column-major, ld = ceil8(m)   (V transposed: columns u contiguous)
//   Wb   n x r  BF16, column-major, ld = ceil8(n)
//   Hb   r x m  BF16, row-major,    ld = ceil8(m)
// V is fixed for the whole job, so both BF16 copies are made once; with
// them, both V-streaming products of an iteration are the same K-major x
// K-major GEMM  D[128 x N] += A[128 x 64] B[N x 64]^T  per 64-wide K block:
//   H-step  W'V:  rows = columns u of V,  A = Vb  tile, B = Wb, K = n
//   W-step  VH':  rows = rows i of V,     A = Vbt tile, B = Hb, K = m
// (src/algorithms/nmf/nmf_multiplicative_euclidian.cpp:37,56, which the
// reference runs as cublasSgemm through DeviceMatrix.h:217-227).
//
// The GEMM is stream-K: every CTA (one per SM) takes an equal contiguous
// share of the (row tile, K block) space, so the work is balanced no matter
// how many row tiles there are.  Its share splits into at most a few
// segments at tile boundaries; each segment's FP32 accumulator is written
// as a partial product slot, and the update kernels (one per half-step) sum
// the slots of a tile in a fixed order, so results are deterministic.
//
// Warp roles in the GEMM (192 threads, one CTA per SM):
//   warp 0      TMA producer (one lane) + TMEM allocation
//   warp 1      tcgen05.mma issuer (one lane)
//   warps 2..5  epilogue: tcgen05.ld of their 32-lane TMEM quarter -> partial slot
// Shared memory holds up to 8 stages of (A 16 KB + B N*128 B), 128-byte
// swizzled as TMA writes them.  TMEM holds two accumulators (N columns
// each) so the epilogue of one segment overlaps the MMAs of the next.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "engine.h"
#include "kernels.h"
#include "tc_ptx.cuh"

namespace gpunmf {
using namespace ptx;

constexpr int kTileM = 128;
constexpr int kBlockK = 64;
constexpr int kGemmThreads = 192;
constexpr int kStageABytes = kTileM * kBlockK * 2;
constexpr int kMaxStages = 8;
constexpr int kSmemBudget = 196 * 1024;  // leaves room for one update-kernel CTA beside a GEMM CTA
constexpr int kMaxRank = 192;  // update kernels keep an r x r Gram plus two r x 33 tiles in shared memory

static inline long long ceil8(long long x) { return (x + 7) / 8 * 8; }
static inline int npad_of(int r) { return (r + 15) / 16 * 16; }

struct SkParams {
    int tiles, kblocks, npad, stages, max_seg;
    int bps;  // 64-wide TMA boxes per stage along K (1 or 2): a stage block covers bps*64 of K
    uint32_t tmem_cols;
    float *partials;
    int *err;
    // Gram reduction done by the epilogue warps: gram_out[e] = sum_z gram_partials[z*E + e]
    const float *gram_partials;
    float *gram_out;
    int gram_count;
    int gram_entries;
};

extern __shared__ __align__(1024) unsigned char tc_dyn_smem[];

__device__ __forceinline__ bool warp_wait(uint64_t *bar, uint32_t parity, int *err, int bit) {
    int ok = 0;
    if ((threadIdx.x & 31) == 0) ok = mbar_wait(bar, parity, err, bit) ? 1 : 0;
    ok = __shfl_sync(0xffffffffu, ok, 0);
    return ok != 0;
}

__global__ void __launch_bounds__(kGemmThreads, 1)
    tc_gemm_sk_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      SkParams p) {
    const uintptr_t base = (reinterpret_cast<uintptr_t>(tc_dyn_smem) + 1023) & ~uintptr_t(1023);
    const int boxB = p.npad * kBlockK * 2;          // one 64-wide B box
    const int stageA = kStageABytes * p.bps, stageB = boxB * p.bps;
    unsigned char *sA = reinterpret_cast<unsigned char *>(base);
    unsigned char *sB = sA + p.stages * stageA;
    uint64_t *full = reinterpret_cast<uint64_t *>(sB + p.stages * stageB);
    uint64_t *empty = full + p.stages;
    uint64_t *tfull = empty + p.stages;  // [2]
    uint64_t *tempty = tfull + 2;        // [2]
    uint64_t *mdone = tempty + 2;        // [1]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mdone + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long T = (long long)p.tiles * p.kblocks;
    const long long lo = (long long)blockIdx.x * T / gridDim.x;
    const long long hi = (long long)(blockIdx.x + 1) * T / gridDim.x;

    if (threadIdx.x == 0) {
        for (int s = 0; s < p.stages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; a++) {
            mbar_init(&tfull[a], 1);
            mbar_init(&tempty[a], 4);
        }
        mbar_init(mdone, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, p.tmem_cols);
        tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        tma_prefetch_desc(&tmA);
        tma_prefetch_desc(&tmB);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // everything above overlaps the previous kernel; its outputs (the B operand, the Gram
    // partials) are read only after this point
    griddep_wait();
    griddep_launch_dependents();

    if (warp == 0) {
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            int armed[kMaxStages];
            for (int s = 0; s < kMaxStages; s++) armed[s] = 0;
            for (long long b = lo; b < hi; b++) {
                const int t = (int)(b / p.kblocks), kb = (int)(b % p.kblocks);
                if (!mbar_wait(&empty[stage], phase ^ 1, p.err, kErrWaitEmpty)) break;
                mbar_arrive_expect_tx(&full[stage], stageA + stageB);
                // adjacent boxes along K: each row's bytes of the stage are requested back to back
                for (int q = 0; q < p.bps; q++)
                    tma_load_2d(sA + stage * stageA + q * kStageABytes, &tmA, (kb * p.bps + q) * kBlockK,
                                t * kTileM, &full[stage]);
                for (int q = 0; q < p.bps; q++)
                    tma_load_2d(sB + stage * stageB + q * boxB, &tmB, (kb * p.bps + q) * kBlockK, 0, &full[stage]);
                armed[stage]++;
                if (++stage == p.stages) {
                    stage = 0;
                    phase ^= 1;
                }
            }
            if (*((volatile int *)p.err) != 0) {
                // error exit: let the copies already issued land before the CTA leaves
                for (int s = 0; s < p.stages; s++)
                    if (armed[s] > 0) mbar_wait_quiet(&full[s], (uint32_t)((armed[s] - 1) & 1));
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16_f32(kTileM, p.npad);
            int stage = 0, acc = 0;
            uint32_t phase = 0, aphase = 0;
            bool ok = true;
            for (long long b = lo; b < hi && ok;) {
                const long long t = b / p.kblocks;
                const long long e = min(hi, (t + 1) * p.kblocks);
                if (!mbar_wait(&tempty[acc], aphase ^ 1, p.err, kErrWaitTmemEmpty)) break;
                tc_fence_after();
                const uint32_t d = tmem + (uint32_t)(acc * p.npad);
                for (long long bb = b; bb < e; bb++) {
                    if (!mbar_wait(&full[stage], phase, p.err, kErrWaitFull)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    for (int q = 0; q < p.bps; q++) {
                        const uint32_t a0 = smem_u32(sA + stage * stageA + q * kStageABytes);
                        const uint32_t b0 = smem_u32(sB + stage * stageB + q * boxB);
#pragma unroll
                        for (int k = 0; k < kBlockK / 16; k++) {
                            tc_mma_f16(d, smem_desc(a0 + k * 32, 16, 1024, 2), smem_desc(b0 + k * 32, 16, 1024, 2),
                                       idesc, (bb > b || q > 0 || k > 0) ? 1u : 0u);
                        }
                    }
                    tc_commit(&empty[stage]);
                    if (++stage == p.stages) {
                        stage = 0;
                        phase ^= 1;
                    }
                }
                if (!ok) break;
                tc_commit(&tfull[acc]);
                if (++acc == 2) {
                    acc = 0;
                    aphase ^= 1;
                }
                b = e;
            }
            // all MMAs issued by this thread have completed once mdone flips
            tc_commit(mdone);
            mbar_wait_quiet(mdone, 0);
        }
    } else {
        // While the first accumulator fills, finish the Gram matrix the update kernel of the
        // previous half-step left as per-CTA partials: this CTA owns entries
        // [c*E/G, (c+1)*E/G); four lanes share an entry and sum the partials in a fixed order.
        if (p.gram_out) {
            const int et = threadIdx.x - 64;  // 0..127
            const long long E = p.gram_entries;
            const long long e0 = (long long)blockIdx.x * E / gridDim.x, e1 = (long long)(blockIdx.x + 1) * E / gridDim.x;
            for (long long eb = e0; eb < e1; eb += 32) {
                const long long e = eb + (et >> 2);
                float s = 0.f;
                if (e < e1) {
                    int z = et & 3;
                    for (; z + 28 < p.gram_count; z += 32) {
                        float v[8];
#pragma unroll
                        for (int q = 0; q < 8; q++) v[q] = p.gram_partials[(size_t)(z + 4 * q) * E + e];
#pragma unroll
                        for (int q = 0; q < 8; q++) s += v[q];
                    }
                    for (; z < p.gram_count; z += 4) s += p.gram_partials[(size_t)z * E + e];
                }
                s += __shfl_xor_sync(0xffffffffu, s, 1);
                s += __shfl_xor_sync(0xffffffffu, s, 2);
                if (e < e1 && (et & 3) == 0) p.gram_out[e] = s;
            }
        }
        const int quarter = warp & 3;
        const int row = quarter * 32 + lane;
        int acc = 0, seg = 0;
        uint32_t aphase = 0;
        for (long long b = lo; b < hi;) {
            const long long t = b / p.kblocks;
            const long long e = min(hi, (t + 1) * p.kblocks);
            if (!warp_wait(&tfull[acc], aphase, p.err, kErrWaitTmemFull)) break;
            tc_fence_after();
            float *dst = p.partials + ((size_t)(blockIdx.x * p.max_seg + seg) * kTileM + row) * p.npad;
            const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * p.npad);
            for (int c = 0; c < p.npad; c += 16) {
                float v[16];
                tmem_ld16(taddr + c, v);
                tmem_ld_wait();
                float4 *d4 = reinterpret_cast<float4 *>(dst + c);
                d4[0] = make_float4(v[0], v[1], v[2], v[3]);
                d4[1] = make_float4(v[4], v[5], v[6], v[7]);
                d4[2] = make_float4(v[8], v[9], v[10], v[11]);
                d4[3] = make_float4(v[12], v[13], v[14], v[15]);
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[acc]);
            if (++acc == 2) {
                acc = 0;
                aphase ^= 1;
            }
            seg++;
            b = e;
        }
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, p.tmem_cols);
    }
}

// ------------------------------------------------------------------------
// conversions
// ------------------------------------------------------------------------
// V (n x m FP32 column-major) -> Vb (ld ldv) and Vbt (= V^T, ld ldvt), 32x32 tiles through shared memory
__global__ void convert_v_kernel(const float *__restrict__ V, int n, int m, __nv_bfloat16 *__restrict__ Vb,
                                 long long ldv, __nv_bfloat16 *__restrict__ Vbt, long long ldvt) {
    __shared__ float tile[32][33];
    const int i0 = blockIdx.x * 32, u0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        int i = i0 + threadIdx.x, u = u0 + k;
        float v = (i < n && u < m) ? V[(long long)u * n + i] : 0.f;
        tile[k][threadIdx.x] = v;
        if (i < n && u < m) Vb[(long long)u * ldv + i] = __float2bfloat16_rn(v);
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        int u = u0 + threadIdx.x, i = i0 + k;
        if (i < n && u < m) Vbt[(long long)i * ldvt + u] = __float2bfloat16_rn(tile[threadIdx.x][k]);
    }
}

// W (n x r FP32 column-major) -> Wb (ld ldw)
__global__ void convert_w_kernel(const float *__restrict__ W, int n, int r, __nv_bfloat16 *__restrict__ Wb,
                                 long long ldw) {
    long long total = (long long)n * r;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        long long a = k / n, i = k % n;
        Wb[a * ldw + i] = __float2bfloat16_rn(W[k]);
    }
}

// H (r x m FP32 column-major) -> Hb (r x m row-major, ld ldh)
__global__ void convert_h_kernel(const float *__restrict__ H, int r, int m, __nv_bfloat16 *__restrict__ Hb,
                                 long long ldh) {
    long long total = (long long)r * m;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        long long u = k / r, a = k % r;
        Hb[a * ldh + u] = __float2bfloat16_rn(H[k]);
    }
}

// ------------------------------------------------------------------------
// update kernel (FP32): the multiplicative rule of nmf_kernels.cu:43-47 (or the
// additive rule of nmf_kernels.cu:31-38) on an
// r x 32 tile X of the factor being updated, with
//   H-step: X = H(:, u0:u0+32),   den = G_W X          (G_W = W'W)
//   W-step: X = W(i0:i0+32, :)',  den = G_H X = (X' G_H)'  (G_H = H H', symmetric)
// The numerator is the sum of the GEMM's partial slots for the tile (fixed
// order).  The kernel writes X (FP32), its BF16 copy for the next GEMM, and
// this CTA's partial Gram X X' (r x r) that the next GEMM's epilogue warps
// reduce.  256 threads as a 16 x 16 grid; RP = r rounded up to 16, so each
// thread owns RP/16 rows of the tile.
// ------------------------------------------------------------------------
constexpr int kUpdCols = 16;  // columns (H-step) or rows (W-step) per CTA; 16 x 16 threads
constexpr int kUpdThreads = 256;
constexpr int kSlotW = 8;  // width of the per-tile slot table (tiles with more slots use the CSR lists)

struct UpdParams {
    float *X;                 // FP32 factor (H column-major r x m, or W column-major n x r)
    __nv_bfloat16 *Xb;        // BF16 copy: element (a, c) at a*ldb + c (Hb row-major / Wb column-major)
    long long ldb;
    long long ldx;            // n for W (W(c,a) at a*n + c); unused for H (H(a,c) at c*r + a)
    const float *G;           // r x r Gram for the denominator
    const float *P;           // GEMM partial slots [slot][128][npad]
    const int *slot_ptr, *slot_list;
    const int *tile_slots;    // [tiles][kSlotW] slot ids, -1 padded; null when a tile has more slots
    float *gram_partials;     // [cta][RP*RP]
    int r, cols, npad;
    float eps;
    int update;               // 0: only write the Gram partials of X (initialisation)
    int additive;             // 1: X = max(0, X + (X / den) (num - den)) (nmf_kernels.cu:31-38)
};

template <int RP, bool IS_W>
__global__ void __launch_bounds__(kUpdThreads) tc_update_kernel(UpdParams p) {
    constexpr int TA = RP / 16;
    constexpr int LDX = kUpdCols + 1;
    extern __shared__ float sm[];
    float *Gs = sm;                  // [RP][RP], zero outside r
    float *Xs = Gs + RP * RP;        // [RP][LDX]  X(a, c)
    float *Ns = Xs + RP * LDX;       // [RP][LDX]  numerators, later the new X as [c][RP + 4]
    const int tid = threadIdx.x;
    const int c0 = blockIdx.x * kUpdCols;
    const int ncol = min(kUpdCols, p.cols - c0);
    const int r = p.r;
    griddep_wait();  // the GEMM's partial slots and Gram are complete
    griddep_launch_dependents();
    // Shared-memory fills: every thread first issues all of its loads (compile-time trip counts,
    // fully unrolled), then stores, so the loads of a thread are in flight together.
    // X tile (zero outside r rows / ncol columns)
    constexpr int XL = RP * kUpdCols / kUpdThreads;
    {
        float xv[XL];
#pragma unroll
        for (int j = 0; j < XL; j++) {
            const int k = tid + j * kUpdThreads;
            if (IS_W) {
                const int a = k / kUpdCols, c = k % kUpdCols;
                xv[j] = (a < r && c < ncol) ? p.X[(long long)a * p.ldx + c0 + c] : 0.f;
            } else {
                const int c = k / RP, a = k % RP;
                xv[j] = (a < r && c < ncol) ? p.X[(long long)(c0 + c) * r + a] : 0.f;
            }
        }
#pragma unroll
        for (int j = 0; j < XL; j++) {
            const int k = tid + j * kUpdThreads;
            if (IS_W) Xs[(k / kUpdCols) * LDX + k % kUpdCols] = xv[j];
            else Xs[(k % RP) * LDX + k / RP] = xv[j];
        }
    }
    if (p.update) {  // G is RP x RP (zero outside r x r: the rows of X beyond r are zero)
        constexpr int GL = RP * RP / kUpdThreads;
        constexpr int GC = GL < 16 ? GL : 16;
#pragma unroll 1
        for (int j0 = 0; j0 < GL; j0 += GC) {
            float gv[GC];
#pragma unroll
            for (int j = 0; j < GC; j++) gv[j] = (j0 + j < GL) ? p.G[tid + (j0 + j) * kUpdThreads] : 0.f;
#pragma unroll
            for (int j = 0; j < GC; j++)
                if (j0 + j < GL) Gs[tid + (j0 + j) * kUpdThreads] = gv[j];
        }
    }
    if (p.update) {
        // numerators: the tile's partial slots summed in slot order.  With the fixed-width slot
        // table every load of every slot is independent, so they are all in flight at once.
        const int tile = c0 / 128, lrow0 = c0 % 128;
        constexpr int PER = kUpdCols * RP / kUpdThreads;
        float acc[PER];
#pragma unroll
        for (int j = 0; j < PER; j++) acc[j] = 0.f;
        if (p.tile_slots) {
            const int4 *ts = reinterpret_cast<const int4 *>(p.tile_slots + (size_t)tile * kSlotW);
            const int4 sa = ts[0], sb = ts[1];
            const int sl[kSlotW] = {sa.x, sa.y, sa.z, sa.w, sb.x, sb.y, sb.z, sb.w};
#pragma unroll
            for (int q = 0; q < kSlotW; q++) {
                if (sl[q] >= 0) {
                    const float *base = p.P + ((size_t)sl[q] * 128 + lrow0) * p.npad;
#pragma unroll
                    for (int j = 0; j < PER; j++) {
                        const int k = tid + j * kUpdThreads, c = k / RP, a = k % RP;
                        if (c < ncol) acc[j] += base[c * p.npad + a];
                    }
                }
            }
        } else {
            const int s0 = p.slot_ptr[tile], s1 = p.slot_ptr[tile + 1];
            for (int q = s0; q < s1; q++) {
                const float *base = p.P + ((size_t)p.slot_list[q] * 128 + lrow0) * p.npad;
#pragma unroll
                for (int j = 0; j < PER; j++) {
                    const int k = tid + j * kUpdThreads, c = k / RP, a = k % RP;
                    if (c < ncol) acc[j] += base[c * p.npad + a];
                }
            }
        }
#pragma unroll
        for (int j = 0; j < PER; j++) {
            const int k = tid + j * kUpdThreads, c = k / RP, a = k % RP;
            Ns[a * LDX + c] = acc[j];
        }
    }
    __syncthreads();
    const int ga = tid & 15, gc = tid >> 4;
    constexpr int CPT = kUpdCols / 16;  // columns per thread
    float *Xn = Ns;  // reused as [c][RP + 4] once the numerators are in registers
    constexpr int LDN = RP + 4;
    if (p.update) {
        // den(a, c) for a in ga*TA.., c in gc*CPT..
        float den[TA][CPT];
#pragma unroll
        for (int i = 0; i < TA; i++)
#pragma unroll
            for (int j = 0; j < CPT; j++) den[i][j] = 0.f;
        for (int b = 0; b < RP; b++) {
            float xb[CPT];
#pragma unroll
            for (int j = 0; j < CPT; j++) xb[j] = Xs[b * LDX + gc * CPT + j];
#pragma unroll
            for (int i = 0; i < TA; i++) {
                float g = Gs[b * RP + ga * TA + i];
#pragma unroll
                for (int j = 0; j < CPT; j++) den[i][j] = fmaf(g, xb[j], den[i][j]);
            }
        }
        float nv[TA][CPT], xv[TA][CPT];
#pragma unroll
        for (int i = 0; i < TA; i++)
#pragma unroll
            for (int j = 0; j < CPT; j++) {
                nv[i][j] = Ns[(ga * TA + i) * LDX + gc * CPT + j];
                xv[i][j] = Xs[(ga * TA + i) * LDX + gc * CPT + j];
            }
        __syncthreads();  // everyone has read Ns and Xs
#pragma unroll
        for (int i = 0; i < TA; i++)
#pragma unroll
            for (int j = 0; j < CPT; j++) {
                int a = ga * TA + i;
                float x = xv[i][j];
                if (a < r && gc * CPT + j < ncol) {  // outside stays 0 (the additive step has no eps)
                    if (p.additive) {
                        x = x + (x / den[i][j]) * (nv[i][j] - den[i][j]);
                        x = x < 0.f ? 0.f : x;
                    } else {
                        x *= nv[i][j] / (den[i][j] + p.eps);
                    }
                }
                Xn[(gc * CPT + j) * LDN + a] = x;
            }
    } else {
        for (int k = tid; k < RP * kUpdCols; k += kUpdThreads) {
            int c = k / RP, a = k % RP;
            Xn[c * LDN + a] = Xs[a * LDX + c];
        }
    }
    __syncthreads();
    if (p.update) {
        if (IS_W) {
            for (int k = tid; k < RP * kUpdCols; k += kUpdThreads) {
                int a = k / kUpdCols, c = k % kUpdCols;
                if (a < r && c < ncol) {
                    float x = Xn[c * LDN + a];
                    p.X[(long long)a * p.ldx + c0 + c] = x;
                    p.Xb[(long long)a * p.ldb + c0 + c] = __float2bfloat16_rn(x);
                }
            }
        } else {
            for (int k = tid; k < RP * kUpdCols; k += kUpdThreads) {
                int c = k / RP, a = k % RP;
                if (a < r && c < ncol) p.X[(long long)(c0 + c) * r + a] = Xn[c * LDN + a];
            }
            for (int k = tid; k < RP * kUpdCols; k += kUpdThreads) {
                int a = k / kUpdCols, c = k % kUpdCols;
                if (a < r && c < ncol) p.Xb[(long long)a * p.ldb + c0 + c] = __float2bfloat16_rn(Xn[c * LDN + a]);
            }
        }
    }
    // partial Gram of the new tile: rows ga*TA.., columns gb*TA.. (columns outside ncol are zero)
    {
        const int gb = tid >> 4;
        float acc[TA][TA];
#pragma unroll
        for (int i = 0; i < TA; i++)
#pragma unroll
            for (int k = 0; k < TA; k++) acc[i][k] = 0.f;
        for (int c = 0; c < kUpdCols; c++) {
            float xa[TA], xb[TA];
#pragma unroll
            for (int i = 0; i < TA; i++) {
                xa[i] = Xn[c * LDN + ga * TA + i];
                xb[i] = Xn[c * LDN + gb * TA + i];
            }
#pragma unroll
            for (int i = 0; i < TA; i++)
#pragma unroll
                for (int k = 0; k < TA; k++) acc[i][k] = fmaf(xa[i], xb[k], acc[i][k]);
        }
        float *out = p.gram_partials + (size_t)blockIdx.x * RP * RP;
#pragma unroll
        for (int i = 0; i < TA; i++)
#pragma unroll
            for (int k = 0; k < TA; k++) out[(ga * TA + i) * RP + gb * TA + k] = acc[i][k];
    }
}

// ------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------
// ========================================================================
// KL rule (nmf_multiplicative_divergence.cpp:29-50, nmf_kernels.cu:247-341):
// fused  S = (W H) block -> R = V / (S + eps) -> numerator += R x factor,
// never materialising W H.  Per 128-row output tile and 64-wide K block:
//   MMA1  D1[128 x 64]  = A1[128 x r] B1[64 x r]^T     (S for the block, in TMEM)
//   epilogue warps: R = V / (D1 + eps) -> BF16, written 128B-swizzled into
//                   shared memory as the next MMA's A operand
//   MMA2  D2[128 x N]  += R[128 x 64] B2[N x 64]^T     (numerator, in TMEM)
//   H-step: rows u; A1 = Hc (H, column-major BF16), B1 = Wr (W, row-major),
//           V tile from Vb, B2 = Wb;                 K = i (rows of V)
//   W-step: rows i; A1 = Wr, B1 = Hc, V tile from Vbt, B2 = Hb;  K = u
// MMA1 of block g+1 is issued before MMA2 of block g so the tensor core
// works while the epilogue warps form R.  Stream-K partition and partial
// slots as in the Euclidean GEMM; the epilogue warps also finish the
// column/row sums (the KL denominators) from the update kernel's partials.
// ========================================================================
struct KlParams {
    int tiles, kblocks, npad, stages, max_seg, nbox;
    uint32_t tmem_cols;
    float eps;
    float *partials;
    int *err;
    const float *sum_partials;  // [count][npad] partial sums of the other factor
    float *sum_out;             // [npad]
    int sum_count;
};

__device__ __forceinline__ uint32_t sw128(int row, int chunk) {
    return (uint32_t)(row * 128 + ((chunk ^ (row & 7)) << 4));
}

constexpr int kKlEpiWarps = 16;  // two groups of 8 (even / odd K blocks); 2 per TMEM lane quarter in a group
constexpr int kKlThreads = 64 + 32 * kKlEpiWarps;  // warp 0 TMA, warp 1 MMA, then the ratio epilogue

__global__ void __launch_bounds__(kKlThreads, 1)
    tc_kl_gemm_kernel(const __grid_constant__ CUtensorMap tmV, const __grid_constant__ CUtensorMap tmA1,
                      const __grid_constant__ CUtensorMap tmB1, const __grid_constant__ CUtensorMap tmB2,
                      KlParams p) {
    const uintptr_t base = (reinterpret_cast<uintptr_t>(tc_dyn_smem) + 1023) & ~uintptr_t(1023);
    const int b1Bytes = p.nbox * 8192, b2Bytes = p.npad * 128;
    const int stageBytes = 16384 + b1Bytes + b2Bytes;
    unsigned char *sStage = reinterpret_cast<unsigned char *>(base);
    unsigned char *sA1 = sStage + p.stages * stageBytes;
    unsigned char *sR = sA1 + p.nbox * 16384;  // [2][16 KB]
    uint64_t *full = reinterpret_cast<uint64_t *>(sR + 2 * 16384);
    uint64_t *empty = full + p.stages;
    uint64_t *a1full = empty + p.stages, *a1empty = a1full + 1;
    uint64_t *d1full = a1empty + 1, *d1empty = d1full + 2;
    uint64_t *rfull = d1empty + 2, *rempty = rfull + 2;
    uint64_t *tfull = rempty + 2, *tempty = tfull + 2;
    uint64_t *mdone = tempty + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mdone + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long T = (long long)p.tiles * p.kblocks;
    const long long lo = (long long)blockIdx.x * T / gridDim.x;
    const long long hi = (long long)(blockIdx.x + 1) * T / gridDim.x;
    auto sV = [&](int st) { return sStage + st * stageBytes; };
    auto sB1 = [&](int st) { return sStage + st * stageBytes + 16384; };
    auto sB2 = [&](int st) { return sStage + st * stageBytes + 16384 + b1Bytes; };

    if (threadIdx.x == 0) {
        for (int s = 0; s < p.stages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(a1full, 1);
        mbar_init(a1empty, 1);
        for (int b = 0; b < 2; b++) {
            mbar_init(&d1full[b], 1);
            mbar_init(&d1empty[b], kKlEpiWarps / 2);  // buffer b is handled by group b
            mbar_init(&rfull[b], kKlEpiWarps / 2);
            mbar_init(&rempty[b], 1);
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], kKlEpiWarps);
        }
        mbar_init(mdone, 1);
        fence_mbar_init();
        tma_prefetch_desc(&tmV);
        tma_prefetch_desc(&tmA1);
        tma_prefetch_desc(&tmB1);
        tma_prefetch_desc(&tmB2);
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, p.tmem_cols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t tD1 = tmem, tD2 = tmem + 128;  // D1: 2 x 64 columns, D2: 2 x npad columns
    griddep_wait();
    griddep_launch_dependents();

    if (warp == 0) {
        if (lane == 0) {
            int stage = 0, seg = 0;
            uint32_t phase = 0;
            for (long long b = lo; b < hi;) {
                const int t = (int)(b / p.kblocks);
                const long long e = min(hi, (long long)(t + 1) * p.kblocks);
                // the factor tile of this row tile (MMA1's A), once per segment
                if (!mbar_wait(a1empty, (uint32_t)((seg & 1) ^ 1), p.err, kErrWaitEmpty)) break;
                mbar_arrive_expect_tx(a1full, (uint32_t)(p.nbox * 16384));
                for (int q = 0; q < p.nbox; q++) tma_load_2d(sA1 + q * 16384, &tmA1, q * 64, t * kTileM, a1full);
                bool ok = true;
                for (long long bb = b; bb < e; bb++) {
                    const int kb = (int)(bb % p.kblocks);
                    if (!mbar_wait(&empty[stage], phase ^ 1, p.err, kErrWaitEmpty)) {
                        ok = false;
                        break;
                    }
                    mbar_arrive_expect_tx(&full[stage], (uint32_t)stageBytes);
                    tma_load_2d(sV(stage), &tmV, kb * kBlockK, t * kTileM, &full[stage]);
                    for (int q = 0; q < p.nbox; q++)
                        tma_load_2d(sB1(stage) + q * 8192, &tmB1, q * 64, kb * kBlockK, &full[stage]);
                    tma_load_2d(sB2(stage), &tmB2, kb * kBlockK, 0, &full[stage]);
                    if (++stage == p.stages) {
                        stage = 0;
                        phase ^= 1;
                    }
                }
                if (!ok) break;
                seg++;
                b = e;
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t id1 = idesc_bf16_f32(kTileM, 64), id2 = idesc_bf16_f32(kTileM, p.npad);
            int stage = 0, seg = 0;
            uint32_t phase = 0;
            long long g = 0;  // global block counter (D1 / R double buffers)
            bool ok = true;
            int prev_stage = 0;
            for (long long b = lo; b < hi && ok;) {
                const int t = (int)(b / p.kblocks);
                const long long e = min(hi, (long long)(t + 1) * p.kblocks);
                const int acc = seg & 1;
                if (!mbar_wait(a1full, (uint32_t)(seg & 1), p.err, kErrWaitFull)) break;
                if (!mbar_wait(&tempty[acc], (uint32_t)(((seg >> 1) & 1) ^ 1), p.err, kErrWaitTmemEmpty)) break;
                tc_fence_after();
                const uint32_t a1 = smem_u32(sA1);
                bool first2 = true;
                for (long long bb = b; bb <= e && ok; bb++) {
                    if (bb < e) {
                        // MMA1 for block g
                        const int db = (int)(g & 1);
                        if (!mbar_wait(&full[stage], phase, p.err, kErrWaitFull) ||
                            !mbar_wait(&d1empty[db], (uint32_t)(((g >> 1) & 1) ^ 1), p.err, kErrWaitTmemEmpty)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t b1 = smem_u32(sB1(stage));
                        for (int k16 = 0; k16 < p.npad / 16; k16++) {
                            const int q = k16 >> 2, w = (k16 & 3) * 32;
                            tc_mma_f16(tD1 + (uint32_t)(db * 64), smem_desc(a1 + q * 16384 + w, 16, 1024, 2),
                                       smem_desc(b1 + q * 8192 + w, 16, 1024, 2), id1, k16 > 0 ? 1u : 0u);
                        }
                        tc_commit(&d1full[db]);
                    }
                    if (bb > b) {
                        // MMA2 for block g-1 (its R is formed by the epilogue warps)
                        const long long gp = g - 1;
                        const int rb = (int)(gp & 1);
                        if (!mbar_wait(&rfull[rb], (uint32_t)((gp >> 1) & 1), p.err, kErrWaitFull)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t ra = smem_u32(sR + rb * 16384), b2 = smem_u32(sB2(prev_stage));
#pragma unroll
                        for (int k = 0; k < 4; k++)
                            tc_mma_f16(tD2 + (uint32_t)(acc * p.npad), smem_desc(ra + k * 32, 16, 1024, 2),
                                       smem_desc(b2 + k * 32, 16, 1024, 2), id2, (first2 && k == 0) ? 0u : 1u);
                        first2 = false;
                        tc_commit(&empty[prev_stage]);
                        tc_commit(&rempty[rb]);
                    }
                    if (bb < e) {
                        prev_stage = stage;
                        if (++stage == p.stages) {
                            stage = 0;
                            phase ^= 1;
                        }
                        g++;
                    }
                }
                if (!ok) break;
                tc_commit(&tfull[acc]);
                tc_commit(a1empty);
                seg++;
                b = e;
            }
            tc_commit(mdone);
            mbar_wait_quiet(mdone, 0);
        }
    } else {
        // finish the denominators (column / row sums of the other factor) from the partials
        if (p.sum_out) {
            const int et = threadIdx.x - 64;  // 0 .. 255
            const int E = p.npad;
            const int e0 = (int)((long long)blockIdx.x * E / gridDim.x), e1 = (int)((long long)(blockIdx.x + 1) * E / gridDim.x);
            for (int eb = e0; eb < e1; eb += kKlEpiWarps * 8) {
                const int ei = eb + (et >> 2);
                float sacc = 0.f;
                if (ei < e1) {
                    int z = et & 3;
                    for (; z + 28 < p.sum_count; z += 32) {
                        float v[8];
#pragma unroll
                        for (int q = 0; q < 8; q++) v[q] = p.sum_partials[(size_t)(z + 4 * q) * E + ei];
#pragma unroll
                        for (int q = 0; q < 8; q++) sacc += v[q];
                    }
                    for (; z < p.sum_count; z += 4) sacc += p.sum_partials[(size_t)z * E + ei];
                }
                sacc += __shfl_xor_sync(0xffffffffu, sacc, 1);
                sacc += __shfl_xor_sync(0xffffffffu, sacc, 2);
                if (ei < e1 && (et & 3) == 0) p.sum_out[ei] = sacc;
            }
        }
        const int quarter = warp & 3;           // TMEM lanes this warp may access
        const int grp = (warp - 2) >> 3;         // group 0 takes even K blocks, group 1 odd ones
        const int part = ((warp - 2) >> 2) & 1;  // which 32 of the block's 64 columns
        const int dpart = (warp - 2) >> 2;       // 0..3: share of the D2 drain
        const float eps_pos = fmaxf(p.eps, 1e-30f);
        const int row = quarter * 32 + lane;
        const uint32_t lane_off = (uint32_t)(quarter * 32) << 16;
        int stage = 0, seg = 0;
        uint32_t sphase = 0;
        long long g = 0;
        for (long long b = lo; b < hi;) {
            const int t = (int)(b / p.kblocks);
            const long long e = min(hi, (long long)(t + 1) * p.kblocks);
            bool ok = true;
            for (long long bb = b; bb < e; bb++) {
                const int db = (int)(g & 1);
                if (db != grp) {  // the other group's block: keep the counters in step
                    if (++stage == p.stages) {
                        stage = 0;
                        sphase ^= 1;
                    }
                    g++;
                    continue;
                }
                if (!warp_wait(&d1full[db], (uint32_t)((g >> 1) & 1), p.err, kErrWaitTmemFull) ||
                    !warp_wait(&full[stage], sphase, p.err, kErrWaitFull) ||
                    !warp_wait(&rempty[db], (uint32_t)(((g >> 1) & 1) ^ 1), p.err, kErrWaitEmpty)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const unsigned char *vt = sV(stage);
                unsigned char *rt = sR + db * 16384;
                // this warp's 32 columns of S for its row: two loads in flight, one wait
                float sv[32];
                {
                    float (&s0)[16] = *reinterpret_cast<float (*)[16]>(&sv[0]);
                    float (&s1)[16] = *reinterpret_cast<float (*)[16]>(&sv[16]);
                    const uint32_t ta = tD1 + (uint32_t)(db * 64 + part * 32) + lane_off;
                    tmem_ld16(ta, s0);
                    tmem_ld16(ta + 16, s1);
                    tmem_ld_wait();
                }
#pragma unroll
                for (int cc = 0; cc < 4; cc++) {  // 16-byte chunks of 8 values
                    const int chunk = part * 4 + cc;
                    const uint4 vraw = *reinterpret_cast<const uint4 *>(vt + sw128(row, chunk));
                    const __nv_bfloat162 *v2 = reinterpret_cast<const __nv_bfloat162 *>(&vraw);
                    uint4 out;
                    __nv_bfloat162 *o2 = reinterpret_cast<__nv_bfloat162 *>(&out);
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        // R is rounded to BF16 (8-bit significand): the approximate division
                        // (2 ulp in FP32) is exact enough.  eps_pos > 0 keeps zero-padded
                        // entries (V = 0, S = 0) at 0.
                        const float2 vf = __bfloat1622float2(v2[q]);
                        const float r0 = __fdividef(vf.x, sv[cc * 8 + 2 * q] + eps_pos);
                        const float r1 = __fdividef(vf.y, sv[cc * 8 + 2 * q + 1] + eps_pos);
                        o2[q] = __floats2bfloat162_rn(r0, r1);
                    }
                    *reinterpret_cast<uint4 *>(rt + sw128(row, chunk)) = out;
                }
                // R written with ordinary stores: make it visible to the tensor core, then hand it over
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                tc_fence_before();
                __syncwarp();
                if (lane == 0) {
                    mbar_arrive(&rfull[db]);
                    mbar_arrive(&d1empty[db]);
                }
                if (++stage == p.stages) {
                    stage = 0;
                    sphase ^= 1;
                }
                g++;
            }
            if (!ok) break;
            const int acc = seg & 1;
            if (!warp_wait(&tfull[acc], (uint32_t)((seg >> 1) & 1), p.err, kErrWaitTmemFull)) break;
            tc_fence_after();
            float *dst = p.partials + ((size_t)(blockIdx.x * p.max_seg + seg) * kTileM + row) * p.npad;
            for (int c = dpart * 16; c < p.npad; c += 64) {  // the four warps of a quarter take turns by 16 columns
                float v[16];
                tmem_ld16(tD2 + (uint32_t)(acc * p.npad) + lane_off + (uint32_t)c, v);
                tmem_ld_wait();
                float4 *d4 = reinterpret_cast<float4 *>(dst + c);
                d4[0] = make_float4(v[0], v[1], v[2], v[3]);
                d4[1] = make_float4(v[4], v[5], v[6], v[7]);
                d4[2] = make_float4(v[8], v[9], v[10], v[11]);
                d4[3] = make_float4(v[12], v[13], v[14], v[15]);
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[acc]);
            seg++;
            b = e;
        }
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, p.tmem_cols);
    }
}

// KL update (nmf_kernels.cu:289,337 with the eps clamp of :104,190): X *= num / max(sum, eps)
// on a 16-wide tile; writes X, its two BF16 copies, and this tile's partial sums over its columns
// (the other half-step's denominator).  The additive KL rule
// (nmf_kernels_additive_divergence.cu:90-104,159-173) needs sum_k f_k (R_k - 1) =
// num - sum_k f_k: the same numerator less the unclamped sum of the other factor.
struct KlUpdParams {
    float *X;
    __nv_bfloat16 *Xb;   // element (a, c) at a*ldb + c   (Hb row-major / Wb column-major)
    long long ldb;
    __nv_bfloat16 *Xr;   // element (a, c) at c*ldr + a   (Hc column-major H / Wr row-major W)
    long long ldr;
    long long ldx;       // W: n
    const float *sums;   // [npad] denominators (before the eps clamp)
    const float *P;
    const int *slot_ptr, *slot_list, *tile_slots;
    float *sum_partials; // [cta][npad]
    int r, cols, npad;
    float eps;
    int update;
    int additive;        // 1: X = max(0, X + (X / max(sum, eps)) (num - sum))
};

template <int RP, bool IS_W>
__global__ void __launch_bounds__(kUpdThreads) tc_kl_update_kernel(KlUpdParams p) {
    constexpr int LDX = kUpdCols + 1;
    __shared__ float Xs[RP * LDX];
    __shared__ float sumS[RP], sumR[RP];
    const int tid = threadIdx.x;
    const int c0 = blockIdx.x * kUpdCols;
    const int ncol = min(kUpdCols, p.cols - c0);
    const int r = p.r;
    griddep_wait();
    griddep_launch_dependents();
    constexpr int XL = RP * kUpdCols / kUpdThreads;
    float xv[XL], acc[XL];
#pragma unroll
    for (int j = 0; j < XL; j++) {
        const int k = tid + j * kUpdThreads;
        if (IS_W) {
            const int a = k / kUpdCols, c = k % kUpdCols;
            xv[j] = (a < r && c < ncol) ? p.X[(long long)a * p.ldx + c0 + c] : 0.f;
        } else {
            const int c = k / RP, a = k % RP;
            xv[j] = (a < r && c < ncol) ? p.X[(long long)(c0 + c) * r + a] : 0.f;
        }
        acc[j] = 0.f;
    }
    if (tid < RP) {
        const float sraw = p.update ? p.sums[tid] : 0.f;
        sumS[tid] = p.update ? fmaxf(sraw, p.eps) : 1.f;
        sumR[tid] = sraw;
    }
    if (p.update) {
        const int tile = c0 / 128, lrow0 = c0 % 128;
        auto add_slot = [&](int sl) {
            const float *bs = p.P + ((size_t)sl * 128 + lrow0) * p.npad;
#pragma unroll
            for (int j = 0; j < XL; j++) {
                const int k = tid + j * kUpdThreads;
                int a, c;
                if (IS_W) { a = k / kUpdCols; c = k % kUpdCols; }
                else      { c = k / RP; a = k % RP; }
                if (c < ncol) acc[j] += bs[c * p.npad + a];
            }
        };
        if (p.tile_slots) {
            const int4 *ts = reinterpret_cast<const int4 *>(p.tile_slots + (size_t)tile * kSlotW);
            const int4 sa = ts[0], sb = ts[1];
            const int sl[kSlotW] = {sa.x, sa.y, sa.z, sa.w, sb.x, sb.y, sb.z, sb.w};
#pragma unroll
            for (int q = 0; q < kSlotW; q++)
                if (sl[q] >= 0) add_slot(sl[q]);
        } else {
            for (int q = p.slot_ptr[tile]; q < p.slot_ptr[tile + 1]; q++) add_slot(p.slot_list[q]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < XL; j++) {
        const int k = tid + j * kUpdThreads;
        int a, c;
        if (IS_W) { a = k / kUpdCols; c = k % kUpdCols; }
        else      { c = k / RP; a = k % RP; }
        float x = xv[j];
        if (p.update && a < r && c < ncol) {
            if (p.additive) {
                x = x + (x / sumS[a]) * (acc[j] - sumR[a]);
                x = x < 0.f ? 0.f : x;
            } else {
                x *= (acc[j] / sumS[a]);
            }
            if (IS_W) p.X[(long long)a * p.ldx + c0 + c] = x;
            else p.X[(long long)(c0 + c) * r + a] = x;
        }
        Xs[a * LDX + c] = x;
    }
    __syncthreads();
    if (p.update) {
        for (int k = tid; k < RP * kUpdCols; k += kUpdThreads) {  // Xb: c fastest
            const int a = k / kUpdCols, c = k % kUpdCols;
            if (a < r && c < ncol) p.Xb[(long long)a * p.ldb + c0 + c] = __float2bfloat16_rn(Xs[a * LDX + c]);
        }
        for (int k = tid; k < RP * kUpdCols; k += kUpdThreads) {  // Xr: a fastest
            const int c = k / RP, a = k % RP;
            if (c < ncol) p.Xr[(long long)(c0 + c) * p.ldr + a] = __float2bfloat16_rn(a < r ? Xs[a * LDX + c] : 0.f);
        }
    }
    if (tid < RP) {
        float sacc = 0.f;
        for (int c = 0; c < kUpdCols; c++) sacc += Xs[tid * LDX + c];
        p.sum_partials[(size_t)blockIdx.x * RP + tid] = sacc;
    }
}

// W (n x r FP32) -> Wr (row-major BF16, ld ldr, zero beyond r); H (r x m) -> Hc (column-major BF16)
__global__ void convert_rowmajor_kernel(const float *__restrict__ X, int rows, int r, long long ldx_rows,
                                        bool x_is_w, __nv_bfloat16 *__restrict__ Xr, long long ldr) {
    long long total = (long long)rows * ldr;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const long long c = k / ldr, a = k % ldr;
        float v = 0.f;
        if (a < r) v = x_is_w ? X[a * ldx_rows + c] : X[c * r + a];
        Xr[k] = __float2bfloat16_rn(v);
    }
}

}  // namespace gpunmf

struct TcGemm {
    CUtensorMap tmA, tmB;
    gpunmf::SkParams p;
    int grid = 0;
    int smem = 0;
    int *slot_ptr = nullptr, *slot_list = nullptr;
    int *tile_slots = nullptr;
};

struct KlGemm {
    CUtensorMap tmV, tmA1, tmB1, tmB2;
    gpunmf::KlParams p;
    int grid = 0, smem = 0;
    int *slot_ptr = nullptr, *slot_list = nullptr, *tile_slots = nullptr;
};

struct TcState {
    __nv_bfloat16 *Vb = nullptr, *Vbt = nullptr, *Wb = nullptr, *Hb = nullptr;
    // KL rule: second BF16 layouts (W row-major, H column-major), denominators and their partials
    __nv_bfloat16 *Wr = nullptr, *Hc = nullptr;
    long long ldr = 0;
    KlGemm kh, kw;
    float *S_w = nullptr, *S_h = nullptr, *SP_w = nullptr, *SP_h = nullptr;
    long long ldv = 0, ldvt = 0, ldw = 0, ldh = 0;
    int npad = 16;
    TcGemm gh, gw;  // H-step (W'V) and W-step (VH')
    float *P_h = nullptr, *P_w = nullptr;
    int *err = nullptr;
    float *G_w = nullptr, *G_h = nullptr;     // W'W and H H', npad x npad
    float *GP_w = nullptr, *GP_h = nullptr;   // per-CTA Gram partials of the update kernels
    int gp_w_count = 0, gp_h_count = 0;
};

namespace gpunmf {

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 2-D BF16 tensor map: dim0 contiguous (extent d0), dim1 with stride ld elements; box {64, box1}, 128B swizzle
static gpunmf_status make_map(CUtensorMap *m, const void *base, uint64_t d0, uint64_t d1, uint64_t ld,
                              uint32_t box1) {
    auto fn = encode_fn();
    if (!fn) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return GPUNMF_ERR_CUDA;
    }
    cuuint64_t dims[2] = {d0, d1};
    cuuint64_t strides[1] = {ld * 2};
    cuuint32_t box[2] = {(cuuint32_t)kBlockK, box1};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return GPUNMF_ERR_CUDA;
    }
    return GPUNMF_OK;
}

static int num_sms() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
            sms = kNumSMsGB300;
    }
    return sms;
}

// stream-K schedule: CTA c covers [c*T/G, (c+1)*T/G); its segments at tile boundaries get slots
// c*max_seg + s.  Builds the per-tile slot lists in CTA order.
static void schedule(int tiles, int kblocks, int G, int *max_seg, std::vector<int> &ptr, std::vector<int> &list) {
    long long T = (long long)tiles * kblocks;
    int ms = 1;
    std::vector<std::vector<int>> per(tiles);
    std::vector<std::vector<int>> segs_tile(G);
    for (int c = 0; c < G; c++) {
        long long lo = (long long)c * T / G, hi = (long long)(c + 1) * T / G;
        int s = 0;
        for (long long b = lo; b < hi;) {
            long long t = b / kblocks, e = std::min(hi, (t + 1) * kblocks);
            segs_tile[c].push_back((int)t);
            s++;
            b = e;
        }
        ms = std::max(ms, s);
    }
    for (int c = 0; c < G; c++)
        for (size_t s = 0; s < segs_tile[c].size(); s++) per[segs_tile[c][s]].push_back(c * ms + (int)s);
    ptr.assign(tiles + 1, 0);
    list.clear();
    for (int t = 0; t < tiles; t++) {
        ptr[t] = (int)list.size();
        for (int x : per[t]) list.push_back(x);
    }
    ptr[tiles] = (int)list.size();
    *max_seg = ms;
}

static gpunmf_status setup_gemm(gpunmf_job *j, TcGemm &g, int rows, int K, int npad, float **partials, int *err) {
    const int tiles = ceil_div(rows, kTileM);
    const int boxB = npad * kBlockK * 2;
    // two 64-wide boxes per stage when at least three such stages fit, else one
    const int bps = (kSmemBudget - 1280) / (2 * (kStageABytes + boxB)) >= 3 ? 2 : 1;
    const int kblocks = ceil_div(K, kBlockK * bps);
    const long long T = (long long)tiles * kblocks;
    g.grid = (int)std::min<long long>(num_sms(), T);
    std::vector<int> ptr, list;
    int max_seg = 1;
    schedule(tiles, kblocks, g.grid, &max_seg, ptr, list);
    bool table_ok = true;
    for (int t = 0; t < tiles; t++)
        if (ptr[t + 1] - ptr[t] > kSlotW) table_ok = false;
    std::vector<int> table;
    if (table_ok) {
        table.assign((size_t)tiles * kSlotW, -1);
        for (int t = 0; t < tiles; t++)
            for (int q = ptr[t]; q < ptr[t + 1]; q++) table[(size_t)t * kSlotW + (q - ptr[t])] = list[q];
    }
    const int stage_bytes = bps * (kStageABytes + boxB);
    int stages = std::min(kMaxStages, (kSmemBudget - 1024 - 256) / stage_bytes);
    g.p.bps = bps;
    g.p.tiles = tiles;
    g.p.kblocks = kblocks;
    g.p.npad = npad;
    g.p.stages = stages;
    g.p.max_seg = max_seg;
    uint32_t cols = 32;
    while (cols < (uint32_t)(2 * npad)) cols <<= 1;
    g.p.tmem_cols = cols;
    g.p.err = err;
    g.smem = 1024 + stages * stage_bytes + (2 * stages + 5) * 8 + 16;
    size_t slots = (size_t)g.grid * max_seg;
    cudaError_t e = job_dev_alloc(j, (void **)partials, slots * kTileM * npad * sizeof(float));
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&g.slot_ptr, ptr.size() * sizeof(int));
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&g.slot_list, std::max<size_t>(1, list.size()) * sizeof(int));
    if (e == cudaSuccess) e = job_h2d(j, g.slot_ptr, ptr.data(), ptr.size() * sizeof(int));
    if (e == cudaSuccess && !list.empty()) e = job_h2d(j, g.slot_list, list.data(), list.size() * sizeof(int));
    if (e == cudaSuccess && table_ok) {
        e = job_dev_alloc(j, (void **)&g.tile_slots, table.size() * sizeof(int));
        if (e == cudaSuccess) e = job_h2d(j, g.tile_slots, table.data(), table.size() * sizeof(int));
    }
    if (e != cudaSuccess) {
        set_error("tensor-core workspace allocation failed: %s", cudaGetErrorString(e));
        cudaGetLastError();
        return GPUNMF_ERR_NOMEM;
    }
    g.p.partials = *partials;
    return GPUNMF_OK;
}

static size_t gemm_partial_bytes(int rows, int K, int npad) {
    const int tiles = ceil_div(rows, kTileM), kblocks = ceil_div(K, kBlockK);
    long long T = (long long)tiles * kblocks;
    int G = (int)std::min<long long>(kNumSMsGB300, T);
    long long per = (T + G - 1) / G;
    long long max_seg = per / kblocks + 2;
    return (size_t)G * max_seg * kTileM * npad * sizeof(float) + (size_t)(tiles + 1 + G * max_seg) * sizeof(int);
}

static cudaError_t set_gemm_smem_once() {
    static std::once_flag once;
    static cudaError_t result = cudaSuccess;
    std::call_once(once, [] {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        result = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (result == cudaSuccess)
            result = cudaFuncSetAttribute(tc_gemm_sk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    });
    return result;
}

static int update_smem_bytes(int rp) {
    int ns = std::max(rp * (kUpdCols + 1), kUpdCols * (rp + 4));
    return (rp * rp + rp * (kUpdCols + 1) + ns) * (int)sizeof(float);
}

template <int RP>
static cudaError_t set_update_smem_rp() {
    cudaError_t e = cudaFuncSetAttribute(tc_update_kernel<RP, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         update_smem_bytes(RP));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(tc_update_kernel<RP, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 update_smem_bytes(RP));
    return e;
}

static cudaError_t set_update_smem(int rp) {
    switch (rp) {
#define CASE(R) \
    case R: return set_update_smem_rp<R>();
        CASE(16) CASE(32) CASE(48) CASE(64) CASE(80) CASE(96) CASE(112) CASE(128) CASE(144) CASE(160) CASE(176)
        CASE(192)
#undef CASE
    }
    return cudaErrorInvalidValue;
}

static cudaError_t launch_update(const UpdParams &u, int rp, bool is_w, cudaStream_t s) {
    const int grid = ceil_div(u.cols, kUpdCols);
    const int smem = update_smem_bytes(rp);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kUpdThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    switch (rp) {
#define CASE(R)                                                                          \
    case R:                                                                              \
        return is_w ? cudaLaunchKernelEx(&cfg, tc_update_kernel<R, true>, u)             \
                    : cudaLaunchKernelEx(&cfg, tc_update_kernel<R, false>, u);
        CASE(16) CASE(32) CASE(48) CASE(64) CASE(80) CASE(96) CASE(112) CASE(128) CASE(144) CASE(160) CASE(176)
        CASE(192)
#undef CASE
    }
    return cudaErrorInvalidValue;
}

static UpdParams update_params_h(gpunmf_job *j, int update) {
    TcState *t = j->tc;
    UpdParams u{};
    u.X = j->H; u.Xb = t->Hb; u.ldb = t->ldh; u.ldx = 0; u.G = t->G_w; u.P = t->P_h;
    u.slot_ptr = t->gh.slot_ptr; u.slot_list = t->gh.slot_list; u.tile_slots = t->gh.tile_slots;
    u.gram_partials = t->GP_h;
    u.r = j->r; u.cols = j->m; u.npad = t->npad; u.eps = j->eps; u.update = update;
    u.additive = rule_is_additive(j->rule);
    return u;
}

static UpdParams update_params_w(gpunmf_job *j, int update) {
    TcState *t = j->tc;
    UpdParams u{};
    u.X = j->W; u.Xb = t->Wb; u.ldb = t->ldw; u.ldx = j->n; u.G = t->G_h; u.P = t->P_w;
    u.slot_ptr = t->gw.slot_ptr; u.slot_list = t->gw.slot_list; u.tile_slots = t->gw.tile_slots;
    u.gram_partials = t->GP_w;
    u.r = j->r; u.cols = j->n; u.npad = t->npad; u.eps = j->eps; u.update = update;
    u.additive = rule_is_additive(j->rule);
    return u;
}

constexpr int kKlSmemBudget = 220 * 1024;
constexpr int kKlMaxRank = 128;

static cudaError_t set_kl_smem_once() {
    static std::once_flag once;
    static cudaError_t result = cudaSuccess;
    std::call_once(once, [] {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        result = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (result == cudaSuccess)
            result = cudaFuncSetAttribute(tc_kl_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    });
    return result;
}

static gpunmf_status setup_kl(gpunmf_job *j, KlGemm &g, int rows, int K, int npad, float **partials, int *err) {
    const int tiles = ceil_div(rows, kTileM);
    const int kblocks = ceil_div(K, kBlockK);
    const long long T = (long long)tiles * kblocks;
    g.grid = (int)std::min<long long>(num_sms(), T);
    std::vector<int> ptr, list;
    int max_seg = 1;
    schedule(tiles, kblocks, g.grid, &max_seg, ptr, list);
    bool table_ok = true;
    for (int t = 0; t < tiles; t++)
        if (ptr[t + 1] - ptr[t] > kSlotW) table_ok = false;
    std::vector<int> table;
    if (table_ok) {
        table.assign((size_t)tiles * kSlotW, -1);
        for (int t = 0; t < tiles; t++)
            for (int q = ptr[t]; q < ptr[t + 1]; q++) table[(size_t)t * kSlotW + (q - ptr[t])] = list[q];
    }
    const int nbox = (npad + 63) / 64;
    const int stage_bytes = 16384 + nbox * 8192 + npad * 128;
    const int fixed = 1024 + nbox * 16384 + 2 * 16384 + 512;
    const int stages = std::min(kMaxStages, (kKlSmemBudget - fixed) / stage_bytes);
    if (stages < 2) {
        set_error("KL tensor-core kernel: rank too large for the shared-memory pipeline");
        return GPUNMF_ERR_UNSUPPORTED;
    }
    g.p.tiles = tiles;
    g.p.kblocks = kblocks;
    g.p.npad = npad;
    g.p.stages = stages;
    g.p.max_seg = max_seg;
    g.p.nbox = nbox;
    g.p.tmem_cols = (128 + 2 * npad) <= 256 ? 256 : 512;
    g.p.eps = j->eps;
    g.p.err = err;
    g.smem = fixed + stages * stage_bytes;
    size_t slots = (size_t)g.grid * max_seg;
    cudaError_t e = job_dev_alloc(j, (void **)partials, slots * kTileM * npad * sizeof(float));
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&g.slot_ptr, ptr.size() * sizeof(int));
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&g.slot_list, std::max<size_t>(1, list.size()) * sizeof(int));
    if (e == cudaSuccess) e = job_h2d(j, g.slot_ptr, ptr.data(), ptr.size() * sizeof(int));
    if (e == cudaSuccess && !list.empty()) e = job_h2d(j, g.slot_list, list.data(), list.size() * sizeof(int));
    if (e == cudaSuccess && table_ok) {
        e = job_dev_alloc(j, (void **)&g.tile_slots, table.size() * sizeof(int));
        if (e == cudaSuccess) e = job_h2d(j, g.tile_slots, table.data(), table.size() * sizeof(int));
    }
    if (e != cudaSuccess) {
        set_error("KL tensor-core workspace allocation failed: %s", cudaGetErrorString(e));
        cudaGetLastError();
        return GPUNMF_ERR_NOMEM;
    }
    g.p.partials = *partials;
    return GPUNMF_OK;
}

static cudaError_t launch_kl_gemm(KlGemm &g, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(g.grid);
    cfg.blockDim = dim3(kKlThreads);
    cfg.dynamicSmemBytes = g.smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, tc_kl_gemm_kernel, g.tmV, g.tmA1, g.tmB1, g.tmB2, g.p);
}

static cudaError_t launch_kl_update(const KlUpdParams &u, int rp, bool is_w, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ceil_div(u.cols, kUpdCols));
    cfg.blockDim = dim3(kUpdThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    switch (rp) {
#define CASE(R)                                                                          \
    case R:                                                                              \
        return is_w ? cudaLaunchKernelEx(&cfg, tc_kl_update_kernel<R, true>, u)          \
                    : cudaLaunchKernelEx(&cfg, tc_kl_update_kernel<R, false>, u);
        CASE(16) CASE(32) CASE(48) CASE(64) CASE(80) CASE(96) CASE(112) CASE(128)
#undef CASE
    }
    return cudaErrorInvalidValue;
}

static KlUpdParams kl_params_h(gpunmf_job *j, int update) {
    TcState *t = j->tc;
    KlUpdParams u{};
    u.X = j->H; u.Xb = t->Hb; u.ldb = t->ldh; u.Xr = t->Hc; u.ldr = t->ldr; u.ldx = 0;
    u.sums = t->S_w; u.P = t->P_h;
    u.slot_ptr = t->kh.slot_ptr; u.slot_list = t->kh.slot_list; u.tile_slots = t->kh.tile_slots;
    u.sum_partials = t->SP_h;
    u.r = j->r; u.cols = j->m; u.npad = t->npad; u.eps = j->eps; u.update = update;
    u.additive = rule_is_additive(j->rule);
    return u;
}

static KlUpdParams kl_params_w(gpunmf_job *j, int update) {
    TcState *t = j->tc;
    KlUpdParams u{};
    u.X = j->W; u.Xb = t->Wb; u.ldb = t->ldw; u.Xr = t->Wr; u.ldr = t->ldr; u.ldx = j->n;
    u.sums = t->S_h; u.P = t->P_w;
    u.slot_ptr = t->kw.slot_ptr; u.slot_list = t->kw.slot_list; u.tile_slots = t->kw.tile_slots;
    u.sum_partials = t->SP_w;
    u.r = j->r; u.cols = j->n; u.npad = t->npad; u.eps = j->eps; u.update = update;
    u.additive = rule_is_additive(j->rule);
    return u;
}

static gpunmf_status tc_create_kl(gpunmf_job *j) {
    TcState *t = j->tc;
    const int n = j->n, m = j->m, r = j->r;
    t->ldr = t->npad;
    const int cw = ceil_div(n, kUpdCols), ch = ceil_div(m, kUpdCols);
    cudaError_t e = job_dev_alloc(j, (void **)&t->Vb, (size_t)t->ldv * m * 2);
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->Vbt, (size_t)t->ldvt * n * 2);
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->Wb, (size_t)t->ldw * r * 2);
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->Hb, (size_t)t->ldh * r * 2);
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->Wr, (size_t)n * t->ldr * 2);
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->Hc, (size_t)m * t->ldr * 2);
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->err, sizeof(int));
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->S_w, t->npad * sizeof(float));
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->S_h, t->npad * sizeof(float));
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->SP_w, (size_t)cw * t->npad * sizeof(float));
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->SP_h, (size_t)ch * t->npad * sizeof(float));
    if (e == cudaSuccess) e = cudaMemsetAsync(t->err, 0, sizeof(int), j->stream);
    if (e != cudaSuccess) {
        set_error("KL tensor-core buffers: %s", cudaGetErrorString(e));
        cudaGetLastError();
        return GPUNMF_ERR_NOMEM;
    }
    gpunmf_status st = setup_kl(j, t->kh, m, n, t->npad, &t->P_h, t->err);
    if (st == GPUNMF_OK) st = setup_kl(j, t->kw, n, m, t->npad, &t->P_w, t->err);
    if (st != GPUNMF_OK) return st;
    t->kh.p.sum_partials = t->SP_w; t->kh.p.sum_out = t->S_w; t->kh.p.sum_count = cw;
    t->kw.p.sum_partials = t->SP_h; t->kw.p.sum_out = t->S_h; t->kw.p.sum_count = ch;
    // H-step: rows u; V tile from Vb, A1 = Hc rows u, B1 = Wr rows i, B2 = Wb
    st = make_map(&t->kh.tmV, t->Vb, n, m, t->ldv, kTileM);
    if (st == GPUNMF_OK) st = make_map(&t->kh.tmA1, t->Hc, r, m, t->ldr, kTileM);
    if (st == GPUNMF_OK) st = make_map(&t->kh.tmB1, t->Wr, r, n, t->ldr, kBlockK);
    if (st == GPUNMF_OK) st = make_map(&t->kh.tmB2, t->Wb, n, r, t->ldw, t->npad);
    // W-step: rows i; V tile from Vbt, A1 = Wr rows i, B1 = Hc rows u, B2 = Hb
    if (st == GPUNMF_OK) st = make_map(&t->kw.tmV, t->Vbt, m, n, t->ldvt, kTileM);
    if (st == GPUNMF_OK) st = make_map(&t->kw.tmA1, t->Wr, r, n, t->ldr, kTileM);
    if (st == GPUNMF_OK) st = make_map(&t->kw.tmB1, t->Hc, r, m, t->ldr, kBlockK);
    if (st == GPUNMF_OK) st = make_map(&t->kw.tmB2, t->Hb, m, r, t->ldh, t->npad);
    if (st != GPUNMF_OK) return st;
    GPUNMF_CUDA_TRY(set_kl_smem_once());
    return GPUNMF_OK;
}

gpunmf_status tc_supported(int rule, int n, int m, int r) {
    (void)n;
    (void)m;
    if (rule_is_kl(rule)) {
        if (r > kKlMaxRank) {
            set_error("BF16 KL path supports r <= %d", kKlMaxRank);
            return GPUNMF_ERR_UNSUPPORTED;
        }
        return GPUNMF_OK;
    }
    if (r > kMaxRank) {
        set_error("BF16 path supports r <= %d", kMaxRank);
        return GPUNMF_ERR_UNSUPPORTED;
    }
    return GPUNMF_OK;
}

void tc_add_sizes(int, int, int, int, size_t *) {}

size_t tc_footprint(int rule, int n, int m, int r) {
    const int npad = npad_of(r);
    if (rule_is_kl(rule)) {
        size_t b = 2 * ((size_t)ceil8(n) * m + (size_t)ceil8(m) * n + (size_t)ceil8(n) * r + (size_t)ceil8(m) * r +
                        (size_t)(n + m) * npad);
        b += gemm_partial_bytes(m, n, npad) + gemm_partial_bytes(n, m, npad);
        b += (size_t)npad * sizeof(float) * (2 + ceil_div(n, kUpdCols) + ceil_div(m, kUpdCols)) + 64;
        return b;
    }
    size_t b = 2 * ((size_t)ceil8(n) * m + (size_t)ceil8(m) * n + (size_t)ceil8(n) * r + (size_t)ceil8(m) * r);
    b += gemm_partial_bytes(m, n, npad) + gemm_partial_bytes(n, m, npad);
    b += (size_t)npad * npad * sizeof(float) * (2 + ceil_div(n, kUpdCols) + ceil_div(m, kUpdCols)) + 64;
    return b;
}

gpunmf_status tc_create(gpunmf_job *j) {
    TcState *t = new (std::nothrow) TcState();
    if (!t) return GPUNMF_ERR_NOMEM;
    j->tc = t;
    const int n = j->n, m = j->m, r = j->r;
    t->npad = npad_of(r);
    t->ldv = ceil8(n);
    t->ldvt = ceil8(m);
    t->ldw = ceil8(n);
    t->ldh = ceil8(m);
    if (rule_is_kl(j->rule)) return tc_create_kl(j);
    cudaError_t e = job_dev_alloc(j, (void **)&t->Vb, (size_t)t->ldv * m * 2);
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->Vbt, (size_t)t->ldvt * n * 2);
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->Wb, (size_t)t->ldw * r * 2);
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->Hb, (size_t)t->ldh * r * 2);
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->err, sizeof(int));
    const size_t rp2 = (size_t)t->npad * t->npad;
    t->gp_w_count = ceil_div(n, kUpdCols);
    t->gp_h_count = ceil_div(m, kUpdCols);
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->G_w, rp2 * sizeof(float));
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->G_h, rp2 * sizeof(float));
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->GP_w, rp2 * t->gp_w_count * sizeof(float));
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->GP_h, rp2 * t->gp_h_count * sizeof(float));
    if (e == cudaSuccess) e = cudaMemsetAsync(t->err, 0, sizeof(int), j->stream);
    if (e != cudaSuccess) {
        set_error("tensor-core buffers: %s", cudaGetErrorString(e));
        cudaGetLastError();
        return GPUNMF_ERR_NOMEM;
    }
    gpunmf_status st = setup_gemm(j, t->gh, m, n, t->npad, &t->P_h, t->err);
    if (st == GPUNMF_OK) st = setup_gemm(j, t->gw, n, m, t->npad, &t->P_w, t->err);
    if (st != GPUNMF_OK) return st;
    // the H-step GEMM finishes W'W from the W-step update's partials, and vice versa
    t->gh.p.gram_partials = t->GP_w;
    t->gh.p.gram_out = t->G_w;
    t->gh.p.gram_count = t->gp_w_count;
    t->gh.p.gram_entries = (int)rp2;
    t->gw.p.gram_partials = t->GP_h;
    t->gw.p.gram_out = t->G_h;
    t->gw.p.gram_count = t->gp_h_count;
    t->gw.p.gram_entries = (int)rp2;
    // H-step: rows = u (columns of V): A = Vb (dim0 i over n, dim1 u over m); B = Wb (dim0 i, dim1 a)
    st = make_map(&t->gh.tmA, t->Vb, n, m, t->ldv, kTileM);
    if (st == GPUNMF_OK) st = make_map(&t->gh.tmB, t->Wb, n, r, t->ldw, t->npad);
    // W-step: rows = i: A = Vbt (dim0 u over m, dim1 i over n); B = Hb (dim0 u, dim1 a)
    if (st == GPUNMF_OK) st = make_map(&t->gw.tmA, t->Vbt, m, n, t->ldvt, kTileM);
    if (st == GPUNMF_OK) st = make_map(&t->gw.tmB, t->Hb, m, r, t->ldh, t->npad);
    if (st != GPUNMF_OK) return st;
    // The attribute is per function, shared by every job in the process: set it once to the
    // device's opt-in maximum, never to one job's size (a concurrent job may need more).
    e = set_gemm_smem_once();
    if (e == cudaSuccess) e = set_update_smem(t->npad);
    if (e != cudaSuccess) {
        set_error("cudaFuncSetAttribute: %s", cudaGetErrorString(e));
        return GPUNMF_ERR_CUDA;
    }
    return GPUNMF_OK;
}

gpunmf_status tc_prepare(gpunmf_job *j) {
    TcState *t = j->tc;
    cudaStream_t s = j->stream;
    dim3 grid(ceil_div(j->n, 32), ceil_div(j->m, 32));
    convert_v_kernel<<<grid, dim3(32, 8), 0, s>>>(j->V, j->n, j->m, t->Vb, t->ldv, t->Vbt, t->ldvt);
    convert_w_kernel<<<std::min(1024, ceil_div((long long)j->n * j->r, 256)), 256, 0, s>>>(j->W, j->n, j->r,
                                                                                          t->Wb, t->ldw);
    convert_h_kernel<<<std::min(1024, ceil_div((long long)j->r * j->m, 256)), 256, 0, s>>>(j->H, j->r, j->m,
                                                                                          t->Hb, t->ldh);
    GPUNMF_CUDA_TRY(cudaGetLastError());
    if (rule_is_kl(j->rule)) {
        convert_rowmajor_kernel<<<std::min(1024, ceil_div((long long)j->n * t->ldr, 256)), 256, 0, s>>>(
            j->W, j->n, j->r, j->n, true, t->Wr, t->ldr);
        convert_rowmajor_kernel<<<std::min(1024, ceil_div((long long)j->m * t->ldr, 256)), 256, 0, s>>>(
            j->H, j->m, j->r, 0, false, t->Hc, t->ldr);
        GPUNMF_CUDA_TRY(cudaGetLastError());
        // column sums of the initial W, finished by the first H-step kernel
        GPUNMF_CUDA_TRY(launch_kl_update(kl_params_w(j, 0), t->npad, true, s));
        return GPUNMF_OK;
    }
    // Gram partials of the initial W, finished by the first H-step GEMM
    GPUNMF_CUDA_TRY(launch_update(update_params_w(j, 0), t->npad, true, s));
    // a rule without an H step: the Gram partials of the (fixed) H, finished by every W-step GEMM
    if (j->rule == GPUNMF_ADDITIVE_EUCLIDEAN_FIXED_H)
        GPUNMF_CUDA_TRY(launch_update(update_params_h(j, 0), t->npad, false, s));
    return GPUNMF_OK;
}

static cudaError_t launch_gemm(TcGemm &g, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(g.grid);
    cfg.blockDim = dim3(kGemmThreads);
    cfg.dynamicSmemBytes = g.smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, tc_gemm_sk_kernel, g.tmA, g.tmB, g.p);
}

gpunmf_status tc_iterate(gpunmf_job *j, bool updateW) {
    TcState *t = j->tc;
    cudaStream_t s = j->stream;
    {
        gpunmf_status st = job_quality_step(j, true);
        if (st != GPUNMF_OK) return st;
    }
    if (rule_is_kl(j->rule)) {
        // H <- H .* [W'(V ./ (WH + eps))] ./ max(colsum W, eps); the kernel also finishes colsum W
        // (additive KL: the same numerator, applied as H + (H / max(colsum W, eps)) (num - colsum W))
        mark_begin(j);
        GPUNMF_CUDA_TRY(launch_kl_gemm(t->kh, s));
        mark_end(j);
        GPUNMF_CUDA_TRY(launch_kl_update(kl_params_h(j, 1), t->npad, false, s));
        j->launches += 2;
        if (!updateW) return GPUNMF_OK;
        // W <- W .* [(V ./ (WH + eps)) H'] ./ max(rowsum H, eps) with the new H
        mark_begin(j);
        GPUNMF_CUDA_TRY(launch_kl_gemm(t->kw, s));
        mark_end(j);
        GPUNMF_CUDA_TRY(launch_kl_update(kl_params_w(j, 1), t->npad, true, s));
        j->launches += 2;
        return GPUNMF_OK;
    }
    // H <- H .* (W'V) ./ (W'W H + eps), or the additive step; the GEMM also finishes W'W
    if (j->rule != GPUNMF_ADDITIVE_EUCLIDEAN_FIXED_H) {
        mark_begin(j);
        GPUNMF_CUDA_TRY(launch_gemm(t->gh, s));
        mark_end(j);
        GPUNMF_CUDA_TRY(launch_update(update_params_h(j, 1), t->npad, false, s));
        j->launches += 2;
    }
    if (!updateW) return GPUNMF_OK;
    // W <- W .* (V H') ./ (W H H' + eps); the GEMM also finishes H H'
    mark_begin(j);
    GPUNMF_CUDA_TRY(launch_gemm(t->gw, s));
    mark_end(j);
    GPUNMF_CUDA_TRY(launch_update(update_params_w(j, 1), t->npad, true, s));
    j->launches += 2;
    return GPUNMF_OK;
}

gpunmf_status tc_check(gpunmf_job *j) {
    if (!j->tc || !j->tc->err) return GPUNMF_OK;
    int e = 0;
    GPUNMF_CUDA_TRY(cudaMemcpy(&e, j->tc->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e != 0) {
        set_error("tensor-core kernel gave up waiting (error bits 0x%x)", e);
        return GPUNMF_ERR_TIMEOUT;
    }
    return GPUNMF_OK;
}

void tc_destroy(gpunmf_job *j) {
    TcState *t = j->tc;
    if (!t) return;
    void *ptrs[] = {t->Vb, t->Vbt, t->Wb, t->Hb, t->P_h, t->P_w, t->err, t->G_h, t->G_w, t->GP_h, t->GP_w,
                    t->gh.slot_ptr, t->gh.slot_list, t->gw.slot_ptr, t->gw.slot_list,
                    t->gh.tile_slots, t->gw.tile_slots, t->Wr, t->Hc, t->S_w, t->S_h, t->SP_w, t->SP_h,
                    t->kh.slot_ptr, t->kh.slot_list, t->kh.tile_slots, t->kw.slot_ptr, t->kw.slot_list,
                    t->kw.tile_slots};
    for (void *p : ptrs) job_dev_free(j, p);
    delete t;
    j->tc = nullptr;
}

}  // namespace gpunmf
