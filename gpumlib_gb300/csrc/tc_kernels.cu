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
// update kernel (FP32): the multiplicative rule of nmf_kernels.cu:43-47 on an
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
                if (a < r) x *= nv[i][j] / (den[i][j] + p.eps);
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
}  // namespace gpunmf

struct TcGemm {
    CUtensorMap tmA, tmB;
    gpunmf::SkParams p;
    int grid = 0;
    int smem = 0;
    int *slot_ptr = nullptr, *slot_list = nullptr;
    int *tile_slots = nullptr;
};

struct TcState {
    __nv_bfloat16 *Vb = nullptr, *Vbt = nullptr, *Wb = nullptr, *Hb = nullptr;
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
    return u;
}

static UpdParams update_params_w(gpunmf_job *j, int update) {
    TcState *t = j->tc;
    UpdParams u{};
    u.X = j->W; u.Xb = t->Wb; u.ldb = t->ldw; u.ldx = j->n; u.G = t->G_h; u.P = t->P_w;
    u.slot_ptr = t->gw.slot_ptr; u.slot_list = t->gw.slot_list; u.tile_slots = t->gw.tile_slots;
    u.gram_partials = t->GP_w;
    u.r = j->r; u.cols = j->n; u.npad = t->npad; u.eps = j->eps; u.update = update;
    return u;
}

gpunmf_status tc_supported(int rule, int n, int m, int r) {
    if (rule != GPUNMF_EUCLIDEAN) {
        set_error("BF16 tensor-core path covers the Euclidean rule");
        return GPUNMF_ERR_UNSUPPORTED;
    }
    if (r > kMaxRank) {
        set_error("BF16 path supports r <= %d", kMaxRank);
        return GPUNMF_ERR_UNSUPPORTED;
    }
    (void)n;
    (void)m;
    return GPUNMF_OK;
}

void tc_add_sizes(int, int, int, int, size_t *) {}

size_t tc_footprint(int rule, int n, int m, int r) {
    (void)rule;
    const int npad = npad_of(r);
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
    // Gram partials of the initial W, finished by the first H-step GEMM
    GPUNMF_CUDA_TRY(launch_update(update_params_w(j, 0), t->npad, true, s));
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
    // H <- H .* (W'V) ./ (W'W H + eps); the GEMM also finishes W'W
    mark_begin(j);
    GPUNMF_CUDA_TRY(launch_gemm(t->gh, s));
    mark_end(j);
    GPUNMF_CUDA_TRY(launch_update(update_params_h(j, 1), t->npad, false, s));
    j->launches += 2;
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
                    t->gh.tile_slots, t->gw.tile_slots};
    for (void *p : ptrs) job_dev_free(j, p);
    delete t;
    j->tc = nullptr;
}

}  // namespace gpunmf
