// BF16 tensor-core path (tcgen05 + TMA) of the Euclidean multiplicative update.
//
// Data layout in HBM (per job, beside the FP32 masters V, W, H):
//   Vb   V as BF16 in 16 KB chunks: chunk (u / 128, i / 64) holds its 128 columns u, each with
//        its 64 rows i contiguous (128 bytes) -- one TMA box, read as one contiguous burst
//   Vbt  V' as BF16 in the same chunking with the roles of i and u swapped
//   (both zero-padded to multiples of 128 in n and m; chunk (t, c) at (t * kb64 + c) * 16 KB,
//   kb64 = the padded K extent / 64)
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
#include <atomic>
#include <climits>
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
    int kb64;  // 64-wide chunks of V per row tile along K (the tiled layout)
    int bps;  // 64-wide TMA boxes per stage along K (1 or 2): a stage block covers bps*64 of K
    uint32_t tmem_cols;
    float *partials;
    int *err;
    long long wait_limit;  // clock64() cycles a bounded wait may last before the kernel gives up
    // Gram reduction done by the epilogue warps: gram_out[e] = sum_z gram_partials[z*E + e]
    const float *gram_partials;
    float *gram_out;
    int gram_count;
    int gram_entries;
    // fused update (kernel template FNP > 0).  Every CTA owns a contiguous slice of the rows of the
    // factor X it updates.  While its tensor pipe streams V, two worker warps assemble the Gram of
    // the other factor from that factor's per-CTA partials (each CTA sums a slice, then all copy
    // the whole), copy the old rows into shared memory and form the denominators X G; after the
    // GEMM, the whole CTA waits until the tiles its rows belong to have all their partial
    // products, sums them, writes the new rows, and leaves its rows' Gram partial for the next
    // kernel.
    float *X;                          // FP32 factor updated: H (r x m) or W (n x r), column-major
    __nv_bfloat16 *Xb;                 // its BF16 copy (Hb row-major / Wb column-major, ld ldb)
    long long ldb;
    int is_w, rows_valid, r, additive; // X is W (rows i) or H (rows u); rows_valid rows
    float eps;
    const int *slot_ptr, *slot_list;   // each tile's slots in K order
    int *tile_cnt, *tile_rd;           // per tile: partial products arrived, readers done (reset by the last)
    const int *tile_readers;           // per tile: how many row chunks read it
    const float *gin_parts;            // [gin_count][npad^2] the other factor's per-CTA Gram partials
    int gin_count;
    float *G_full;                     // npad^2: the complete Gram of the other factor, assembled here
    int *red_cnt;                      // [2]: Gram slices published, CTAs done reading (last resets)
    float *gp;                         // [grid][npad^2] this kernel's per-CTA partials of the new factor
    // quality sample folded into an H-step (kernels with quality warps): sum V log10(WH + eps) - WH of
    // the factors this launch starts from (nmf_kernels_quality.cu:35), WH formed block by block
    float qeps;
    double *qpartial;                  // [grid] per-CTA partials
    int *qdone;                        // CTAs done (the last sums the partials in CTA order, resets it)
    float *qout, *qout_host;           // the value: device word, and the pinned read-back word (or null)
};

extern __shared__ __align__(1024) unsigned char tc_dyn_smem[];

// Wait of a whole warp on an mbarrier phase: lane 0 waits suspended in the barrier (a spinning lane
// would take issue slots from the warps that work meanwhile), the others at the shuffle.
__device__ __forceinline__ bool warp_wait(uint64_t *bar, uint32_t parity, int *err, int bit, long long limit) {
    int ok = 0;
    if ((threadIdx.x & 31) == 0) ok = mbar_wait_sleep(bar, parity, err, bit, limit) ? 1 : 0;
    ok = __shfl_sync(0xffffffffu, ok, 0);
    return ok != 0;
}

__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

// barrier of the four epilogue warps that also ORs a per-thread flag: every thread gets the same
// answer at the same barrier, so the warps leave a loop together
__device__ __forceinline__ bool epi_bar_or(bool v) {
    unsigned r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, 1, 128, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((unsigned)v)
        : "memory");
    return r != 0;
}

// Shared memory the fused update needs beside the stage ring (bytes): the Gram for the
// denominator, a 64-row staging tile, a flag word and the slot lists of two tiles.
constexpr int kFusedSlots = 15;  // slots per tile the fused update handles (more: the separate update kernel)
__host__ __device__ constexpr int fused_gram_floats(int np) { return np * np > 64 * np ? np * np : 64 * np; }
// Per-CTA Gram partials are stored packed: entry (i, k), i <= k, at k (k + 1) / 2 + i, a partial every
// tri_stride(np) floats.  The CTA that sums entries [u0, u1) of every partial then reads one contiguous
// run of each.
__host__ __device__ constexpr int tri_stride(int np) { return (np * (np + 1) / 2 + 3) / 4 * 4; }
__host__ __device__ constexpr int fused_smem_bytes(int np) {
    // the Gram area also holds a chunk's denominators (64 x np)
    return np == 0 ? 0 : fused_gram_floats(np) * 4 + 64 * (np + 4) * 4 + 16 + 2 * (kFusedSlots + 1) * 4 + 64;
}

// The fused update: while V streams, two worker warps (64 threads, named barrier 2) prepare it
// beside the four warps that drain TMEM; after the GEMM, all 256 threads of the CTA finish it.
// Chunks of up to 64 rows are staged as sX[64][NP + 4].  Thread layouts (NT threads):
//   products:  RPT x APT block of (row, a) per thread
//   Gram:      NPT entries (row ga of the Gram, columns gb0..) per thread
template <int NP, int NT>
struct FusedLayout {
    static constexpr int LDX = NP + 4;
    static constexpr int APT = 8, AG = NP / APT, RG = NT / AG, RPT = 64 / RG;
    static constexpr int TPA = NT / NP, NPT = NP / TPA;
    static constexpr int SL = 64 * NP / NT;   // staged values per thread
    static_assert(AG * RG == NT && RG * RPT == 64 && TPA * NP == NT && NPT % 4 == 0, "fused layout");
};

__device__ __forceinline__ void wk_bar() { asm volatile("bar.sync 2, 64;" ::: "memory"); }

// N consecutive floats from shared memory, N * 4-byte aligned (N = 4: one 16-byte load)
template <int N>
__device__ __forceinline__ void lds_vec(const float *src, float (&v)[N]) {
    if constexpr (N == 4) {
        const float4 t = *reinterpret_cast<const float4 *>(src);
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    } else if constexpr (N == 2) {
        const float2 t = *reinterpret_cast<const float2 *>(src);
        v[0] = t.x; v[1] = t.y;
    } else {
#pragma unroll
        for (int i = 0; i < N; i++) v[i] = src[i];
    }
}

// rows [row0, row0 + nrows) (nrows <= 64) of a factor into sX[rho][a], zero elsewhere, up to 32
// loads in flight per thread.  w_layout: W(i, a) at a*ld + i (threads along i); else H(a, u) at
// u*r + a (threads along a).
template <int NP, int NT>
__device__ __forceinline__ void stage_rows(const float *__restrict__ X, int w_layout, long long ld, int r,
                                           long long row0, int nrows, float *sX, int tid) {
    using L = FusedLayout<NP, NT>;
    constexpr int B = L::SL < 32 ? L::SL : 32;
#pragma unroll 1
    for (int k0 = 0; k0 < L::SL; k0 += B) {
        float v[B];
#pragma unroll
        for (int q = 0; q < B; q++) {
            const int k = tid + (k0 + q) * NT;
            if (w_layout) {
                const int a = k >> 6, rho = k & 63;
                v[q] = (rho < nrows && a < r) ? X[(long long)a * ld + row0 + rho] : 0.f;
            } else {
                const int rho = k / NP, a = k % NP;
                v[q] = (rho < nrows && a < r) ? X[(row0 + rho) * r + a] : 0.f;
            }
        }
#pragma unroll
        for (int q = 0; q < B; q++) {
            const int k = tid + (k0 + q) * NT;
            if (w_layout) sX[(k & 63) * L::LDX + (k >> 6)] = v[q];
            else sX[(k / NP) * L::LDX + k % NP] = v[q];
        }
    }
}

// The same staging as asynchronous copies (cp.async, zero-filled outside the rows / r), issued and
// committed but not waited for: all of them are in flight at once, which matters while V streams.
// vec16: H rows copied 16 bytes at a time (r a multiple of 4, so every row starts 16-byte aligned).
__device__ __forceinline__ void cp_async4(float *dst, const float *src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(valid ? 4 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async16(float *dst, const float *src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <int NP, int NT>
__device__ __forceinline__ void stage_rows_async(const float *__restrict__ X, int w_layout, long long ld, int r,
                                                 long long row0, int nrows, float *sX, int tid, bool vec16) {
    using L = FusedLayout<NP, NT>;
    if (!w_layout && vec16) {
        for (int k = tid; k < 64 * NP / 4; k += NT) {
            const int rho = k / (NP / 4), a = (k % (NP / 4)) * 4;
            const bool ok = rho < nrows && a < r;
            cp_async16(sX + rho * L::LDX + a, ok ? X + (row0 + rho) * r + a : X, ok);
        }
    } else {
        for (int k = tid; k < 64 * NP; k += NT) {
            int rho, a;
            const float *src;
            if (w_layout) {
                a = k >> 6; rho = k & 63;
                src = X + (long long)a * ld + row0 + rho;
            } else {
                rho = k / NP; a = k % NP;
                src = X + (row0 + rho) * r + a;
            }
            const bool ok = rho < nrows && a < r;
            cp_async4(sX + rho * L::LDX + a, ok ? src : X, ok);
        }
    }
    cp_async_commit();
}

// den = X G for the staged chunk (b in order, fmaf(G[b][a], x[b], den) as the separate update
// kernel forms them), then stored over the Gram area as sD[rho][a] after `bar` (every thread is
// done reading G)
template <int NP, int NT, class Bar>
__device__ __forceinline__ void chunk_denominators(const float *sX, float *sG, int tid, Bar bar) {
    using L = FusedLayout<NP, NT>;
    const int a0 = (tid % L::AG) * L::APT, r0 = (tid / L::AG) * L::RPT;
    float den[L::RPT][L::APT];
#pragma unroll
    for (int k = 0; k < L::RPT; k++)
#pragma unroll
        for (int q = 0; q < L::APT; q++) den[k][q] = 0.f;
#pragma unroll 1
    for (int b = 0; b < NP; b += 4) {
        float4 xr[L::RPT];
#pragma unroll
        for (int k = 0; k < L::RPT; k++) xr[k] = *reinterpret_cast<const float4 *>(sX + (r0 + k) * L::LDX + b);
#pragma unroll
        for (int jb = 0; jb < 4; jb++) {
            float gv[L::APT];
#pragma unroll
            for (int cc = 0; cc < L::APT / 4; cc++) {
                const float4 g4 = *reinterpret_cast<const float4 *>(sG + (b + jb) * NP + a0 + 4 * cc);
                gv[4 * cc] = g4.x; gv[4 * cc + 1] = g4.y; gv[4 * cc + 2] = g4.z; gv[4 * cc + 3] = g4.w;
            }
#pragma unroll
            for (int k = 0; k < L::RPT; k++) {
                const float xv = jb == 0 ? xr[k].x : jb == 1 ? xr[k].y : jb == 2 ? xr[k].z : xr[k].w;
#pragma unroll
                for (int q = 0; q < L::APT; q++) den[k][q] = fmaf(gv[q], xv, den[k][q]);
            }
        }
    }
    bar();
#pragma unroll
    for (int k = 0; k < L::RPT; k++)
#pragma unroll
        for (int cc = 0; cc < L::APT / 4; cc++)
            *reinterpret_cast<float4 *>(sG + (r0 + k) * NP + a0 + 4 * cc) =
                make_float4(den[k][4 * cc], den[k][4 * cc + 1], den[k][4 * cc + 2], den[k][4 * cc + 3]);
}

// Entry u of the upper triangle of an NP x NP Gram, column by column: (i, k) with i <= k,
// u = k (k + 1) / 2 + i.
__device__ __forceinline__ int2 tri_entry(int u) {
    int k = (int)((sqrtf(8.f * (float)u + 1.f) - 1.f) * 0.5f);
    if ((k + 1) * (k + 2) / 2 <= u) k++;
    if (k * (k + 1) / 2 > u) k--;
    return make_int2(u - k * (k + 1) / 2, k);
}

// Prologue of the fused update (the two worker warps, while V streams).  The complete Gram of the
// other factor is assembled from that factor's per-CTA partials: this CTA sums a slice of the
// upper triangle over the partials in their order (so the result does not depend on which CTA
// does it) and writes both mirror entries.  The partials are packed (tri_stride), so this CTA's
// slice of one partial is one contiguous run and a warp's loads of it share sectors (the run was
// scattered over the partial's columns before: 8.7 us for this phase at 8192 x 8192, r = 64, under
// the V stream); once every CTA has published its slice (grid-wide counter, bounded wait) the
// whole Gram is copied in.  Meanwhile the old rows of this CTA's first
// chunk are copied in; then the chunk's denominators (left in sG as sD).  All copies are
// cp.async, so they are in flight together while the stream holds HBM.
template <int NP>
__device__ __forceinline__ void fused_prologue(const SkParams &pr, int wt, float *sG, float *sX, int *sflag) {
    constexpr int E = NP * NP, U = NP * (NP + 1) / 2, CAP = fused_gram_floats(NP);
    const int c = blockIdx.x, G = gridDim.x, P = pr.gin_count;
    const long long x0 = (long long)c * pr.rows_valid / G, x1 = (long long)(c + 1) * pr.rows_valid / G;
    stage_rows_async<NP, 64>(pr.X, pr.is_w, pr.rows_valid, pr.r, x0, (int)min(64LL, x1 - x0), sX, wt,
                             (pr.r & 3) == 0);
    const int u0 = (int)((long long)c * U / G), u1 = (int)((long long)(c + 1) * U / G);
    const int per = CAP / P;  // entries whose partials fit the staging area at once (P <= 152)
    for (int ub = u0; ub < u1; ub += per) {
        const int nb = min(per, u1 - ub);
        for (int k = wt; k < nb * P; k += 64) {  // sG[q * nb + j]: entry ub + j of partial q
            const int q = k / nb, j = k - q * nb;
            cp_async4(sG + k, pr.gin_parts + (size_t)q * tri_stride(NP) + ub + j, true);
        }
        cp_async_commit();
        cp_async_wait_all();
        wk_bar();
        for (int j = wt; j < nb; j += 64) {
            float sum = 0.f;
            for (int q = 0; q < P; q++) sum += sG[q * nb + j];
            const int2 ik = tri_entry(ub + j);
            pr.G_full[ik.x * NP + ik.y] = sum;
            pr.G_full[ik.y * NP + ik.x] = sum;
        }
        wk_bar();
    }
    cp_async_wait_all();
    wk_bar();  // the slice's Gram entries are written by both warps: one release publishes them
    if (wt == 0) {
        red_release_add(pr.red_cnt, 1);
        sflag[2] = flag_wait_ge(pr.red_cnt, G, pr.err, kErrWaitGram, pr.wait_limit) ? 1 : 0;
    }
    wk_bar();
    if (!sflag[2]) return;  // the error word is set: the tail is skipped
    for (int k = wt; k < E / 4; k += 64) cp_async16(sG + 4 * k, pr.G_full + 4 * k, true);
    cp_async_commit();
    cp_async_wait_all();
    wk_bar();
    // count this CTA past the wait; the answer is used after the denominators (the atomic's round
    // trip overlaps them): the last CTA resets both counters
    const int passed = wt == 0 ? atomicAdd(pr.red_cnt + 1, 1) : 0;
    chunk_denominators<NP, 64>(sX, sG, wt, wk_bar);
    if (wt == 0 && passed == G - 1) {
        pr.red_cnt[1] = 0;
        atomicExch(pr.red_cnt, 0);
    }
}

// Tail of the fused update (all 256 threads, after the GEMM): per chunk of this CTA's rows, wait
// until the chunk's tiles have all their partial products, sum them in K order,
// X_new = X num / (den + eps) or max(0, X + X / den (num - den)), write X and its BF16 copy and
// add the new rows to this CTA's Gram partial, which the next kernel sums with the other CTAs'.
// barrier of the NT threads that run the fused tail: the whole CTA, or (SUBSET) its first NT
// threads (named barrier 4)
template <int NT, bool SUBSET>
__device__ __forceinline__ void tail_sync() {
    if constexpr (SUBSET) asm volatile("bar.sync 4, %0;" ::"n"(NT) : "memory");
    else __syncthreads();
}

// The Gram partial of a chunk at rank 64: the lower triangle of the 64 x 64 block (with its
// diagonal) split over NT threads (256 or 512) so that no thread forms products above the
// diagonal.  The 120 off-diagonal 4 x 4 blocks are cut into 4 x 2 pieces (NT = 256) or 2 x 2 pieces
// (NT = 512); each diagonal block's 10 entries into two pieces of five, all in the last warp: piece
// s of block d holds the 2 x 2 lower triangle of columns 4d + 2s, 4d + 2s + 1 and the entries
// (4d + 2, 4d + s), (4d + 3, 4d + s).  With NT = 256 the last warp also takes blocks 112-119 in
// 2 x 2 pieces.  Every entry is summed over the rows in order, as with any other split.
template <int NT>
struct TriGram64 {
    static_assert(NT == 256 || NT == 512, "rank-64 Gram split");
    static constexpr int kOffRows = NT == 256 ? 4 : 2;  // rows of an off-diagonal piece (2 columns)
    bool last;           // the last warp: a diagonal piece (and with NT = 256 a 2 x 2 piece)
    int ra, cb;          // off-diagonal piece: rows ra.., columns cb, cb + 1
    int dd, ds;          // diagonal piece: block dd, half ds
    float off[kOffRows][2];
    float dg[5];
    __device__ __forceinline__ static void block_of(int ob, int &bi, int &bj) {  // ob-th block below the diagonal
        bi = 1;
        while (bi * (bi + 1) / 2 <= ob) bi++;
        bj = ob - bi * (bi - 1) / 2;
    }
    __device__ __forceinline__ void init(int tid) {
        const int warp = tid >> 5, lane = tid & 31;
        last = warp == NT / 32 - 1;
        int ob, piece, bi, bj;
        if (NT == 256 && last) {
            ob = 112 + (lane >> 2);
            piece = lane & 3;
        } else {
            ob = NT == 256 ? tid >> 1 : tid >> 2;
            piece = NT == 256 ? tid & 1 : tid & 3;
        }
        block_of(ob, bi, bj);
        if (NT == 256 && !last) {
            ra = 4 * bi;
            cb = 4 * bj + 2 * piece;
        } else {
            ra = 4 * bi + 2 * (piece >> 1);
            cb = 4 * bj + 2 * (piece & 1);
        }
        dd = lane >> 1;
        ds = lane & 1;
#pragma unroll
        for (int i = 0; i < kOffRows; i++) off[i][0] = off[i][1] = 0.f;
#pragma unroll
        for (int i = 0; i < 5; i++) dg[i] = 0.f;
    }
    // rows [0, nr) of the staged chunk (row stride ldx floats)
    __device__ __forceinline__ void add_rows(const float *sX, int ldx, int nr) {
        if (!last) {
#pragma unroll 4
            for (int rr = 0; rr < nr; rr++) {
                float xa[kOffRows], xb[2];
                lds_vec<kOffRows>(sX + rr * ldx + ra, xa);
                lds_vec<2>(sX + rr * ldx + cb, xb);
#pragma unroll
                for (int i = 0; i < kOffRows; i++) {
                    off[i][0] = fmaf(xa[i], xb[0], off[i][0]);
                    off[i][1] = fmaf(xa[i], xb[1], off[i][1]);
                }
            }
        } else {
            const int c0 = 4 * dd;
#pragma unroll 4
            for (int rr = 0; rr < nr; rr++) {
                const float *row = sX + rr * ldx;
                float u[2], x23[2];
                lds_vec<2>(row + c0 + 2 * ds, u);
                lds_vec<2>(row + c0 + 2, x23);
                const float w = row[c0 + ds];
                dg[0] = fmaf(u[0], u[0], dg[0]);
                dg[1] = fmaf(u[1], u[0], dg[1]);
                dg[2] = fmaf(u[1], u[1], dg[2]);
                dg[3] = fmaf(x23[0], w, dg[3]);
                dg[4] = fmaf(x23[1], w, dg[4]);
                if constexpr (NT == 256) {
                    float xa[2], xb[2];
                    lds_vec<2>(row + ra, xa);
                    lds_vec<2>(row + cb, xb);
#pragma unroll
                    for (int i = 0; i < 2; i++) {
                        off[i][0] = fmaf(xa[i], xb[0], off[i][0]);
                        off[i][1] = fmaf(xa[i], xb[1], off[i][1]);
                    }
                }
            }
        }
    }
    // entry (a, b), b <= a, at a (a + 1) / 2 + b of the packed partial
    __device__ __forceinline__ void store(float *gpc) const {
        const int nrows = last ? 2 : kOffRows;
        if (!last || NT == 256) {
#pragma unroll
            for (int i = 0; i < kOffRows; i++)
                if (i < nrows) {
                    float *dst = gpc + (ra + i) * (ra + i + 1) / 2 + cb;
                    dst[0] = off[i][0];
                    dst[1] = off[i][1];
                }
        }
        if (last) {
            const int a0 = 4 * dd + 2 * ds, c = 4 * dd + ds, a2 = 4 * dd + 2;
            gpc[a0 * (a0 + 1) / 2 + a0] = dg[0];
            gpc[(a0 + 1) * (a0 + 2) / 2 + a0] = dg[1];
            gpc[(a0 + 1) * (a0 + 2) / 2 + a0 + 1] = dg[2];
            gpc[a2 * (a2 + 1) / 2 + c] = dg[3];
            gpc[(a2 + 1) * (a2 + 2) / 2 + c] = dg[4];
        }
    }
};

template <int NP, int NT = 256, bool SUBSET = false>
__device__ __forceinline__ void fused_tail(const SkParams &pr, int tid, float *sG, float *sX, int *sflag, int *sSl) {
    using L = FusedLayout<NP, NT>;
    constexpr int E = NP * NP;
    // Gram partial: a GB x GB2 block per thread (16 x TB threads)
    constexpr int TB = NT / 16, GB = NP / 16, GB2 = NP / TB;
    constexpr int kMaxBatch = 4; // slots whose loads are issued together
    const int c = blockIdx.x, G = gridDim.x;
    float *const X = pr.X;
    __nv_bfloat16 *const Xb = pr.Xb;
    const float *const partials = pr.partials;
    int *const err = pr.err;
    const long long ldb = pr.ldb;
    const int is_w = pr.is_w, r = pr.r, rows = pr.rows_valid, additive = pr.additive;
    const float eps = pr.eps;
    const long long x0 = (long long)c * rows / G, x1 = (long long)(c + 1) * rows / G;
    const int a0 = (tid % L::AG) * L::APT, r0 = (tid / L::AG) * L::RPT;
    const int ga0 = (tid / TB) * GB, gb0 = (tid % TB) * GB2;
    float *const gpc = pr.gp + (size_t)c * tri_stride(NP);
    const float *sD = sG;
    auto bar = [] { tail_sync<NT, SUBSET>(); };
    float gacc[GB][GB2];  // other ranks
#pragma unroll
    for (int i = 0; i < GB; i++)
#pragma unroll
        for (int k = 0; k < GB2; k++) gacc[i][k] = 0.f;
    TriGram64<NT> tg;  // rank 64
    if constexpr (NP == 64) tg.init(tid);
#pragma unroll 1
    for (long long xb = x0; xb < x1; xb += 64) {
        const int nr = (int)min(64LL, x1 - xb);
        if (xb != x0) {  // later chunks (more than 64 rows per CTA): stage, reload G, denominators
            tail_sync<NT, SUBSET>();
            stage_rows<NP, NT>(X, is_w, rows, r, xb, nr, sX, tid);
            for (int k = tid; k < E / 4; k += NT)
                reinterpret_cast<float4 *>(sG)[k] = __ldcg(reinterpret_cast<const float4 *>(pr.G_full) + k);
            tail_sync<NT, SUBSET>();
            chunk_denominators<NP, NT>(sX, sG, tid, bar);
        }
        const int t0 = (int)(xb / kTileM), t1 = (int)((xb + nr - 1) / kTileM);  // t1 <= t0 + 1
        // once past the waits, count this CTA as a reader of the chunk's tiles; the answers are used
        // at the end of the chunk, where the last reader of a tile resets its counters (every
        // reader is past its wait by then; the slots themselves stay until the next launch)
        int rd0 = 0, rd1 = 0, last0 = -1, last1 = -1;
        if (tid == 0) {
            last0 = pr.tile_readers[t0] - 1;
            if (t1 > t0) last1 = pr.tile_readers[t1] - 1;
            bool ok = true;
            for (int t = t0; t <= t1 && ok; t++)
                ok = flag_wait_ge(pr.tile_cnt + t, pr.slot_ptr[t + 1] - pr.slot_ptr[t], err, kErrWaitTile,
                                  pr.wait_limit);
            if (ok) {
                rd0 = atomicAdd(pr.tile_rd + t0, 1);
                if (t1 > t0) rd1 = atomicAdd(pr.tile_rd + t1, 1);
            }
            *sflag = ok ? 1 : 0;
        }
        // the chunk's slot lists (at most kFusedSlots per tile, checked on the host), fetched by two
        // threads of the second warp while thread 0 waits (they are fixed for the launch)
        if (tid >= 32 && tid < 34 && t0 + tid - 32 <= t1) {
            const int u = tid - 32, t = t0 + u, q0 = pr.slot_ptr[t], ns = pr.slot_ptr[t + 1] - q0;
            sSl[u * (kFusedSlots + 1)] = ns;
            for (int q = 0; q < ns; q++) sSl[u * (kFusedSlots + 1) + 1 + q] = pr.slot_list[q0 + q];
        }
        tail_sync<NT, SUBSET>();      // thread 0's acquire loads and this barrier order the slot reads below
        if (!*sflag) return;  // uniform
        float num[L::RPT][L::APT];
#pragma unroll
        for (int k = 0; k < L::RPT; k++)
#pragma unroll
            for (int q = 0; q < L::APT; q++) num[k][q] = 0.f;
        {
            int tk[L::RPT], lr[L::RPT];
#pragma unroll
            for (int k = 0; k < L::RPT; k++) {
                const long long grow = xb + r0 + k;
                tk[k] = (int)(grow / kTileM) - t0;
                lr[k] = (int)(grow % kTileM);
            }
            const int nsmax = max(sSl[0], t1 > t0 ? sSl[kFusedSlots + 1] : 0);
            for (int q0 = 0; q0 < nsmax; q0 += kMaxBatch) {  // the loads of up to kMaxBatch slots together
                float4 v[kMaxBatch][L::RPT][2];
#pragma unroll
                for (int qq = 0; qq < kMaxBatch; qq++)
#pragma unroll
                    for (int k = 0; k < L::RPT; k++) {
                        const int *sl = sSl + tk[k] * (kFusedSlots + 1);
                        const int q = q0 + qq;
                        if (r0 + k < nr && q < sl[0]) {
                            const float4 *src = reinterpret_cast<const float4 *>(
                                partials + ((size_t)sl[1 + q] * kTileM + lr[k]) * NP + a0);
                            v[qq][k][0] = __ldcg(src);
                            v[qq][k][1] = __ldcg(src + 1);
                        } else {
                            v[qq][k][0] = v[qq][k][1] = make_float4(0.f, 0.f, 0.f, 0.f);
                        }
                    }
#pragma unroll
                for (int qq = 0; qq < kMaxBatch; qq++)  // slots in K order
#pragma unroll
                    for (int k = 0; k < L::RPT; k++) {
                        num[k][0] += v[qq][k][0].x; num[k][1] += v[qq][k][0].y;
                        num[k][2] += v[qq][k][0].z; num[k][3] += v[qq][k][0].w;
                        num[k][4] += v[qq][k][1].x; num[k][5] += v[qq][k][1].y;
                        num[k][6] += v[qq][k][1].z; num[k][7] += v[qq][k][1].w;
                    }
            }
        }
#pragma unroll
        for (int k = 0; k < L::RPT; k++)
#pragma unroll
            for (int q = 0; q < L::APT; q++) {
                const int a = a0 + q;
                const float xv = sX[(r0 + k) * L::LDX + a], d = sD[(r0 + k) * NP + a], nv = num[k][q];
                float v = 0.f;
                if (r0 + k < nr && a < r) {
                    if (additive) {
                        v = xv + (xv / d) * (nv - d);
                        v = v < 0.f ? 0.f : v;
                    } else {
                        v = xv * (nv / (d + eps));
                    }
                }
                num[k][q] = v;
            }
        tail_sync<NT, SUBSET>();  // old rows and partial slots read by every thread
#pragma unroll
        for (int k = 0; k < L::RPT; k++)
#pragma unroll
            for (int cc = 0; cc < L::APT / 4; cc++)
                *reinterpret_cast<float4 *>(sX + (r0 + k) * L::LDX + a0 + 4 * cc) =
                    make_float4(num[k][4 * cc], num[k][4 * cc + 1], num[k][4 * cc + 2], num[k][4 * cc + 3]);
        tail_sync<NT, SUBSET>();
        // column-order writes (W, and both factors' BF16 copies): a warp step covers 32 rows of four
        // columns, lane l row l, the column rotating with l / 8 and the step, so the reads of the
        // staged rows (row stride 4 banks mod 32) fall in 32 distinct banks
#pragma unroll 4
        for (int kk = 0; kk < L::SL; kk++) {
            const int k = tid + kk * NT;
            const int lane = k & 31, st = (k >> 5) & 3, patch = k >> 7;
            const int ac = 4 * (patch >> 1) + (((lane >> 3) + st) & 3), rc = 32 * (patch & 1) + lane;
            if (is_w) {
                if (rc < nr && ac < r) {
                    const float v = sX[rc * L::LDX + ac];
                    X[(long long)ac * rows + xb + rc] = v;
                    Xb[(long long)ac * ldb + xb + rc] = __float2bfloat16_rn(v);
                }
            } else {
                const int rho = k / NP, a = k % NP;
                if (rho < nr && a < r) X[(xb + rho) * r + a] = sX[rho * L::LDX + a];
                if (rc < nr && ac < r) Xb[(long long)ac * ldb + xb + rc] = __float2bfloat16_rn(sX[rc * L::LDX + ac]);
            }
        }
        // this chunk's new rows into this CTA's Gram partial, rows in order
        if constexpr (NP == 64) {
            tg.add_rows(sX, L::LDX, nr);
        } else {
#pragma unroll 4
            for (int rr = 0; rr < nr; rr++) {
                float xa[GB], xb2[GB2];
                lds_vec<GB>(sX + rr * L::LDX + ga0, xa);
                lds_vec<GB2>(sX + rr * L::LDX + gb0, xb2);
#pragma unroll
                for (int i = 0; i < GB; i++)
#pragma unroll
                    for (int k = 0; k < GB2; k++) gacc[i][k] = fmaf(xa[i], xb2[k], gacc[i][k]);
            }
        }
        if (tid == 0) {
            if (rd0 == last0) {
                pr.tile_cnt[t0] = 0;
                pr.tile_rd[t0] = 0;
            }
            if (t1 > t0 && rd1 == last1) {
                pr.tile_cnt[t1] = 0;
                pr.tile_rd[t1] = 0;
            }
        }
    }
    // this CTA's partial, packed (tri_stride): the thread's block holds G(ga, gb) for ga in
    // [ga0, ga0 + GB), gb in [gb0, gb0 + GB2); those with gb <= ga are entry (gb, ga), at
    // ga (ga + 1) / 2 + gb
    if constexpr (NP == 64) {
        tg.store(gpc);
    } else if (ga0 + GB - 1 >= gb0) {
#pragma unroll
        for (int i = 0; i < GB; i++) {
            const int ga = ga0 + i;
            float *dst = gpc + ga * (ga + 1) / 2;
#pragma unroll
            for (int k = 0; k < GB2; k++)
                if (gb0 + k <= ga) dst[gb0 + k] = gacc[i][k];
        }
    }
}

// Gram partials of a factor for the first fused kernel: CTA c over rows [c*rows/G, (c+1)*rows/G),
// the row partition the fused kernels use, so the partials match the ones they leave.
template <int NP>
__global__ void __launch_bounds__(64) gram_partials_kernel(const float *__restrict__ X, int w_layout, int rows,
                                                            int r, float *__restrict__ out) {
    using L = FusedLayout<NP, 64>;
    __shared__ __align__(16) float sX[64 * L::LDX];
    const int wt = threadIdx.x, c = blockIdx.x, G = gridDim.x;
    const long long x0 = (long long)c * rows / G, x1 = (long long)(c + 1) * rows / G;
    const int ga = wt / L::TPA, gb0 = (wt % L::TPA) * L::NPT;
    float gacc[L::NPT];
#pragma unroll
    for (int k = 0; k < L::NPT; k++) gacc[k] = 0.f;
    for (long long xb = x0; xb < x1; xb += 64) {
        const int nr = (int)min(64LL, x1 - xb);
        __syncthreads();
        stage_rows<NP, 64>(X, w_layout, rows, r, xb, nr, sX, wt);
        __syncthreads();
        for (int rr = 0; rr < nr; rr++) {
            const float xa = sX[rr * L::LDX + ga];
#pragma unroll
            for (int k = 0; k < L::NPT; k++) gacc[k] = fmaf(xa, sX[rr * L::LDX + gb0 + k], gacc[k]);
        }
    }
    for (int k = 0; k < L::NPT; k++)  // packed (tri_stride): entry (gb, ga), gb <= ga
        if (gb0 + k <= ga) out[(size_t)c * tri_stride(NP) + ga * (ga + 1) / 2 + gb0 + k] = gacc[k];
}

// threads of the GEMM: producer, MMA issuer, four TMEM-draining warps, with a fused update two
// worker warps, and with a folded quality sample eight quality warps (warps 8-15)
__host__ __device__ constexpr int gemm_threads(int fnp, bool qf = false) {
    return (fnp ? kGemmThreads + 64 : kGemmThreads) + (qf ? 256 : 0);
}
constexpr int kQfWarps = 8;
constexpr uint32_t kQfTmemS = 128;  // TMEM column of the first of the 128-column S buffers
// S buffers (TMEM, 128 columns each, after the two accumulators): three, so that the MMA of a block's S
// waits for the quality warps' read of the S three blocks back, and the stage that S MMA reads (its W
// tile) is held that much less (two: the sampling H-step's stream waited on the quality warps)
constexpr int kQfSBufs = 3;

// The hardware's approximate base-2 logarithm (lg2.approx.ftz.f32): its argument s + eps is at
// least eps >= 1e-30 (s >= 0), a normal float, so flushing subnormals changes nothing.
__device__ __forceinline__ float lg2_approx(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// QF: the H-step also samples the quality of the factors it starts from (the value
// NMF::DetermineQualityImprovement reads, nmf_base.h:70-89), on the V tiles it streams anyway:
// per block (128 columns u of V x 128 rows i) one more MMA forms S = H' W over the block
// (A: the tile's columns of H, from Hb, MN-major, loaded once per segment; B: the stage's W tile,
// read MN-major -- the same bytes the main product reads K-major), into one of two 128-column TMEM
// buffers, and eight quality warps (two per TMEM lane quarter, 64 columns each) add
// v log2(s + eps) and s over S and the stage's V tile before the stage is released (copying the V
// tile into TMEM instead, so the stage could go as soon as its MMAs were done, measured slower:
// 93.3 vs 89.5 us per iteration with the sample).  The per-CTA sums are combined by the last CTA in
// CTA order, so the value is deterministic.
template <int FNP, bool QF = false>
__global__ void __launch_bounds__(gemm_threads(FNP, QF), 1)
    tc_gemm_sk_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      const __grid_constant__ CUtensorMap tmQ, SkParams p) {
    const uintptr_t base = (reinterpret_cast<uintptr_t>(tc_dyn_smem) + 1023) & ~uintptr_t(1023);
    const int boxB = p.npad * kBlockK * 2;          // one 64-wide B box
    const int stageA = kStageABytes * p.bps, stageB = boxB * p.bps;
    const int qslot = QF ? 2 * boxB : 0;            // two 64-column boxes of H's tile columns
    unsigned char *sA = reinterpret_cast<unsigned char *>(base);
    unsigned char *sB = sA + p.stages * stageA;
    unsigned char *sQ = sB + p.stages * stageB;     // [2][qslot] (QF)
    uint64_t *full = reinterpret_cast<uint64_t *>(sQ + 2 * qslot);
    uint64_t *empty = full + p.stages;
    uint64_t *tfull = empty + p.stages;  // [2]
    uint64_t *tempty = tfull + 2;        // [2]
    uint64_t *mdone = tempty + 2;        // [1]
    uint64_t *qfull = mdone + 1;         // QF: [2] H tile loaded, [2] free, [2] S ready, [2] S drained
    uint64_t *qempty = qfull + 2, *sfull = qempty + 2, *sempty = sfull + kQfSBufs;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(QF ? sempty + kQfSBufs : mdone + 1);
    // fused-update areas (FNP > 0): Gram, 64-row staging tile, flag
    float *sG = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(tmem_slot + 4) + 15) & ~uintptr_t(15));
    float *sX = sG + fused_gram_floats(FNP);
    int *sflag = reinterpret_cast<int *>(sX + 64 * (FNP + 4));
    int *sSl = sflag + 4;
    double *qred = reinterpret_cast<double *>(sSl + 2 * (kFusedSlots + 1));  // QF: [2][kQfWarps]
    const uint32_t tcols = QF ? 512u : p.tmem_cols;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long T = (long long)p.tiles * p.kblocks;
    const long long lo = (long long)blockIdx.x * T / gridDim.x;
    const long long hi = (long long)(blockIdx.x + 1) * T / gridDim.x;

    if (threadIdx.x == 0) {
        for (int s = 0; s < p.stages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], QF ? 1 + kQfWarps : 1);  // the MMAs, and the quality warps' V reads
        }
        for (int a = 0; a < 2; a++) {
            mbar_init(&tfull[a], 1);
            mbar_init(&tempty[a], 4);
            if constexpr (QF) {
                mbar_init(&qfull[a], 1);
                mbar_init(&qempty[a], 1);
            }
        }
        if constexpr (QF) {
            for (int a = 0; a < kQfSBufs; a++) {
                mbar_init(&sfull[a], 1);
                mbar_init(&sempty[a], kQfWarps);
            }
        }
        mbar_init(mdone, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, tcols);
        tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        tma_prefetch_desc(&tmA);
        tma_prefetch_desc(&tmB);
        if constexpr (QF) tma_prefetch_desc(&tmQ);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // everything above overlaps the previous kernel; its outputs (the B operand, the Gram
    // partials, the factors) are read only after griddepcontrol.wait.  V is not one of them, so
    // the producer requests the first stages' V boxes before it waits.

    if (warp == 0) {
        if (lane == 0) {
            const uint64_t vpol = l2_policy_evict_first();  // V is read once per launch
            int stage = 0;
            uint32_t phase = 0;
            int armed[kMaxStages];
            for (int s = 0; s < kMaxStages; s++) armed[s] = 0;
            // QF: the H tile of each segment (the columns u of its row tile), into slot qs
            int qcur = -1, qs = 0, qloads = 0, qarmed[2] = {0, 0};
            uint32_t qph = 0;
            bool qok = true;
            auto load_q = [&](int t) {
                if constexpr (QF) {
                    if (t == qcur || !qok) return;
                    if (qloads >= 2 && !mbar_wait(&qempty[qs], qph ^ 1, p.err, kErrWaitEmpty, p.wait_limit)) {
                        qok = false;
                        return;
                    }
                    mbar_arrive_expect_tx(&qfull[qs], (uint32_t)qslot);
                    for (int q = 0; q < 2; q++)
                        tma_load_2d(sQ + qs * qslot + q * boxB, &tmQ, t * kTileM + q * 64, 0, &qfull[qs]);
                    qarmed[qs]++;
                    qloads++;
                    qcur = t;
                    if (++qs == 2) {
                        qs = 0;
                        qph ^= 1;
                    }
                } else {
                    (void)t;
                }
            };
            const int pre = (int)min((long long)p.stages, hi - lo);  // fresh stages: no empty wait
            for (int i = 0; i < pre; i++) {
                const long long b = lo + i;
                const int t = (int)(b / p.kblocks), kb = (int)(b % p.kblocks);
                mbar_arrive_expect_tx(&full[i], stageA + stageB);
                for (int q = 0; q < p.bps; q++)
                    tma_load_3d_hint(sA + i * stageA + q * kStageABytes, &tmA, 0, 0, t * p.kb64 + kb * p.bps + q,
                                     &full[i], vpol);
            }
            griddep_wait();
            griddep_launch_dependents();
            for (int i = 0; i < pre; i++) {
                const int kb = (int)((lo + i) % p.kblocks);
                load_q((int)((lo + i) / p.kblocks));
                for (int q = 0; q < p.bps; q++)
                    tma_load_2d(sB + i * stageB + q * boxB, &tmB, (kb * p.bps + q) * kBlockK, 0, &full[i]);
                armed[i]++;
            }
            stage = pre == p.stages ? 0 : pre;
            phase = pre == p.stages ? 1u : 0u;
            for (long long b = lo + pre; b < hi; b++) {
                const int t = (int)(b / p.kblocks), kb = (int)(b % p.kblocks);
                load_q(t);
                if (!qok || !mbar_wait(&empty[stage], phase ^ 1, p.err, kErrWaitEmpty, p.wait_limit)) break;
                mbar_arrive_expect_tx(&full[stage], stageA + stageB);
                // adjacent boxes along K: each row's bytes of the stage are requested back to back
                for (int q = 0; q < p.bps; q++)
                    tma_load_3d_hint(sA + stage * stageA + q * kStageABytes, &tmA, 0, 0, t * p.kb64 + kb * p.bps + q,
                                     &full[stage], vpol);
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
                for (int s = 0; s < 2; s++)
                    if (qarmed[s] > 0) mbar_wait_quiet(&qfull[s], (uint32_t)((qarmed[s] - 1) & 1));
            }
        } else {
            griddep_wait();
            griddep_launch_dependents();
        }
    } else if (warp == 1) {
        griddep_wait();
        griddep_launch_dependents();
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16_f32(kTileM, p.npad);
            // S = H' W over a block: both operands MN-major, the second 64 of M / N one box further
            const uint32_t idesc_q = idesc_bf16_f32(kTileM, 128) | kIdescAMnMajor | kIdescBMnMajor;
            int stage = 0, acc = 0, qs = 0, sb = 0;
            uint32_t phase = 0, aphase = 0, qph = 0, sph = 0;
            bool ok = true;
            for (long long b = lo; b < hi && ok;) {
                const long long t = b / p.kblocks;
                const long long e = min(hi, (t + 1) * p.kblocks);
                if (!mbar_wait(&tempty[acc], aphase ^ 1, p.err, kErrWaitTmemEmpty, p.wait_limit)) break;
                if constexpr (QF) {
                    if (!mbar_wait(&qfull[qs], qph, p.err, kErrWaitFull, p.wait_limit)) break;
                }
                tc_fence_after();
                const uint32_t d = tmem + (uint32_t)(acc * p.npad);
                for (long long bb = b; bb < e; bb++) {
                    if (!mbar_wait(&full[stage], phase, p.err, kErrWaitFull, p.wait_limit)) {
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
                    if constexpr (QF) {
                        if (!mbar_wait(&sempty[sb], sph ^ 1, p.err, kErrWaitTmemEmpty, p.wait_limit)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t qa = smem_u32(sQ + qs * qslot), qb = smem_u32(sB + stage * stageB);
                        for (int k16 = 0; k16 < p.npad / 16; k16++)
                            tc_mma_f16(tmem + kQfTmemS + (uint32_t)(sb * 128), smem_desc(qa + k16 * 2048, boxB, 1024, 2),
                                       smem_desc(qb + k16 * 2048, boxB, 1024, 2), idesc_q, k16 > 0 ? 1u : 0u);
                        tc_commit(&sfull[sb]);
                        if (++sb == kQfSBufs) {
                            sb = 0;
                            sph ^= 1;
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
                if constexpr (QF) {
                    tc_commit(&qempty[qs]);  // the segment's H tile is free once its MMAs complete
                    if (++qs == 2) {
                        qs = 0;
                        qph ^= 1;
                    }
                }
                b = e;
            }
            // all MMAs issued by this thread have completed once mdone flips
            tc_commit(mdone);
            mbar_wait_quiet(mdone, 0);
        }
    } else if (warp < 6) {
        griddep_wait();
        griddep_launch_dependents();
        // While the first accumulator fills, finish the Gram matrix the update kernel of the
        // previous half-step left as per-CTA partials: this CTA owns entries
        // [c*E/G, (c+1)*E/G); four lanes share an entry and sum the partials in a fixed order.
        if (FNP == 0 && p.gram_out) {
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
            const bool ok = warp_wait(&tfull[acc], aphase, p.err, kErrWaitTmemFull, p.wait_limit);
            if constexpr (FNP > 0) {
                if (epi_bar_or(!ok)) break;  // the fused epilogue's barriers need all four warps
            } else if (!ok) {
                break;
            }
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
            if constexpr (FNP > 0) {
                // this segment's partial product is out: count it on its tile (the four warps'
                // stores are ordered before the barrier, one release publishes them)
                epi_bar();
                if (threadIdx.x == 64) red_release_add(&p.tile_cnt[t], 1);
            }
            seg++;
            b = e;
        }
    } else if constexpr (FNP > 0) {
      if (warp < 8) {
        griddep_wait();
        griddep_launch_dependents();
        fused_prologue<FNP>(p, threadIdx.x - kGemmThreads, sG, sX, sflag);  // warps 6 and 7
      } else if constexpr (QF) {
        griddep_wait();
        griddep_launch_dependents();
        // quality warps 8-15: warp w reads TMEM lane quarter w % 4 (the block's rows u), columns
        // 64 * half .. of S (rows i of the block, the stage's V box `half`)
        const int qw = warp - 8, quarter = warp & 3, half = qw >> 2;
        const int row = quarter * 32 + lane;
        const float eps = fmaxf(p.qeps, 1e-30f);
        double dlog = 0.0, ds = 0.0;
        int stage = 0, sb = 0;
        uint32_t phase = 0, sph = 0;
        for (long long b = lo; b < hi; b++) {
            if (!warp_wait(&sfull[sb], sph, p.err, kErrWaitTmemFull, p.wait_limit)) break;
            if (!warp_wait(&full[stage], phase, p.err, kErrWaitFull, p.wait_limit)) break;  // the V tile
            tc_fence_after();
            const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + kQfTmemS + (uint32_t)(sb * 128 + half * 64);
            const unsigned char *vrow = sA + stage * stageA + half * kStageABytes + row * 128;
            // four independent sums each (the chain of one would be the epilogue's critical path)
            float plog[4] = {0.f, 0.f, 0.f, 0.f}, ps[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int c2 = 0; c2 < 2; c2++) {  // 32 columns at a time
                float sv[32];
                {
                    float (&s0)[16] = *reinterpret_cast<float (*)[16]>(&sv[0]);
                    float (&s1)[16] = *reinterpret_cast<float (*)[16]>(&sv[16]);
                    tmem_ld16(taddr + (uint32_t)(c2 * 32), s0);
                    tmem_ld16(taddr + (uint32_t)(c2 * 32 + 16), s1);
                }
                uint4 raw[4];
#pragma unroll
                for (int k = 0; k < 4; k++)
                    raw[k] = *reinterpret_cast<const uint4 *>(vrow + (((c2 * 4 + k) ^ (row & 7)) << 4));
                tmem_ld_wait();
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const __nv_bfloat162 *h2 = reinterpret_cast<const __nv_bfloat162 *>(&raw[k]);
#pragma unroll
                    for (int e2 = 0; e2 < 4; e2++) {
                        const float2 vv = __bfloat1622float2(h2[e2]);
                        const int j = 8 * k + 2 * e2;
                        plog[e2] = fmaf(vv.x, lg2_approx(sv[j] + eps), plog[e2]);
                        plog[e2] = fmaf(vv.y, lg2_approx(sv[j + 1] + eps), plog[e2]);
                        ps[e2] += sv[j];
                        ps[e2] += sv[j + 1];
                    }
                }
            }
            dlog += (double)((plog[0] + plog[1]) + (plog[2] + plog[3]));
            ds += (double)((ps[0] + ps[1]) + (ps[2] + ps[3]));
            tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&sempty[sb]);
                mbar_arrive(&empty[stage]);
            }
            if (++stage == p.stages) {
                stage = 0;
                phase ^= 1;
            }
            if (++sb == kQfSBufs) {
                sb = 0;
                sph ^= 1;
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            dlog += __shfl_down_sync(0xffffffffu, dlog, off);
            ds += __shfl_down_sync(0xffffffffu, ds, off);
        }
        if (lane == 0) {
            qred[qw] = dlog;
            qred[kQfWarps + qw] = ds;
        }
        asm volatile("bar.sync 5, 256;" ::: "memory");  // the eight quality warps
        if (qw == 0) {
            if (lane == 0) {
                double l = 0.0, sm = 0.0;
                for (int w = 0; w < kQfWarps; w++) {
                    l += qred[w];
                    sm += qred[kQfWarps + w];
                }
                p.qpartial[blockIdx.x] = 0.30102999566398120 * l - sm;  // log10(x) = log2(x) log10(2)
                // publishes this partial; the last CTA's add also acquires every other CTA's
                reinterpret_cast<volatile int *>(qred)[0] = atom_acq_rel_add(p.qdone, 1) == (int)gridDim.x - 1;
            }
            __syncwarp();
            if (reinterpret_cast<volatile int *>(qred)[0]) {
                // the last CTA: the partials summed in CTA order (lane-strided, then a fixed tree)
                double q = 0.0;
                for (int c = lane; c < (int)gridDim.x; c += 32) q += __ldcg(p.qpartial + c);
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) q += __shfl_down_sync(0xffffffffu, q, off);
                if (lane == 0) {
                    p.qout[0] = (float)q;
                    if (p.qout_host) {
                        p.qout_host[0] = (float)q;
                        __threadfence_system();
                    }
                    *p.qdone = 0;
                }
            }
        }
    }
    }
    __syncthreads();
    if constexpr (FNP > 0) {
        // every role is done: the threads finish the update (skipped, uniformly, after an error) --
        // with quality warps at rank 64 all 512 (half the rows per thread: nothing spills at the
        // 128 registers a 512-thread CTA allows), at rank 32 the first 256
        const bool go = __syncthreads_and(*((volatile int *)p.err) == 0);
        if constexpr (QF && FNP == 64) {
            if (go) fused_tail<FNP, 512, false>(p, threadIdx.x, sG, sX, sflag, sSl);
        } else if constexpr (QF) {
            if (go && threadIdx.x < 256) fused_tail<FNP, 256, true>(p, threadIdx.x, sG, sX, sflag, sSl);
        } else {
            if (go) fused_tail<FNP, 256, false>(p, threadIdx.x, sG, sX, sflag, sSl);
        }
        __syncthreads();
    }
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, tcols);
    }
}

// ------------------------------------------------------------------------
// quality on the tensor cores (BF16 jobs): sum V log10(WH + eps) - WH over all of V
// (src/cuda/nmf/nmf_kernels_quality.cu:35, the value NMF::DetermineQualityImprovement samples),
// with WH formed 128 x 128 at a time by tcgen05 from K-major BF16 copies of W (row-major) and H
// (column-major) and never stored; V is streamed as BF16 from its transposed copy, two 128-byte
// swizzled boxes per tile, so a thread reads its row's values 16 bytes at a time without bank
// conflicts.  Warp 0 loads (TMA), warp 1 issues the
// MMAs (double-buffered TMEM), sixteen warps (four per TMEM lane quarter, 32 columns each) read
// the accumulator and the V tile and add up sum v log2(s + eps) and sum s separately, FP32 per
// tile row, FP64 across tiles; quality = log10(2) * the first - the second.  Rows and columns
// beyond n and m read zeros (TMA fill), which add 0.
// ------------------------------------------------------------------------
constexpr int kQEpiWarps = 16;
constexpr int kQThreads = 64 + 32 * kQEpiWarps;
constexpr int kQTile = 128;
constexpr int kQVBytes = kQTile * kQTile * 2;


struct QParams {
    int tiles_i, tiles_u, npad, stages;
    int kb64;         // 64-wide chunks of V' per 128-row tile along u
    float eps;
    double *partial;  // [grid]
    int *err;
    long long wait_limit;
    int *done;        // CTAs finished (the last one sums the partials and resets it)
    float *out;       // the quality (device)
    float *out_host;  // the job's pinned read-back word, written directly where the device can (else null)
};

__global__ void __launch_bounds__(kQThreads, 1)
    tc_quality_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      const __grid_constant__ CUtensorMap tmV, QParams p) {
    const uintptr_t base = (reinterpret_cast<uintptr_t>(tc_dyn_smem) + 1023) & ~uintptr_t(1023);
    // factor tiles MN-major, straight from the BF16 copies the iterations keep (Wb column-major: rows i
    // contiguous; Hb row-major: columns u contiguous): two 64-wide boxes of npad K-rows each
    const int boxBytes = p.npad * 128;
    const int stageBytes = 4 * boxBytes + kQVBytes;
    unsigned char *ring = reinterpret_cast<unsigned char *>(base);
    uint64_t *full = reinterpret_cast<uint64_t *>(ring + p.stages * stageBytes);
    uint64_t *empty = full + p.stages;
    uint64_t *tfull = empty + p.stages;  // [2]
    uint64_t *tempty = tfull + 2;        // [2]
    uint64_t *mdone = tempty + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mdone + 1);
    double *red = reinterpret_cast<double *>(tmem_slot + 2);  // [2][kQEpiWarps], 8-byte aligned
    auto sA = [&](int st) { return ring + st * stageBytes; };
    auto sB = [&](int st) { return ring + st * stageBytes + 2 * boxBytes; };
    auto sV = [&](int st) { return reinterpret_cast<const __nv_bfloat16 *>(ring + st * stageBytes + 4 * boxBytes); };

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int T = p.tiles_i * p.tiles_u;
    if (threadIdx.x == 0) {
        for (int st = 0; st < p.stages; st++) {
            mbar_init(&full[st], 1);
            mbar_init(&empty[st], 1 + kQEpiWarps);  // the MMAs (A, B) and the epilogue warps (V)
        }
        for (int a = 0; a < 2; a++) {
            mbar_init(&tfull[a], 1);
            mbar_init(&tempty[a], kQEpiWarps);
        }
        mbar_init(mdone, 1);
        fence_mbar_init();
        tma_prefetch_desc(&tmA);
        tma_prefetch_desc(&tmB);
        tma_prefetch_desc(&tmV);
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, 2 * kQTile);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // the factors are read only after the kernel that wrote them has completed (griddepcontrol.wait);
    // V is not written by it, so the producer requests the first stages' V tiles before it waits

    if (warp == 0) {
        if (lane == 0) {
            int st = 0;
            uint32_t ph = 0;
            int armed[4] = {0, 0, 0, 0};
            const uint64_t vpol = l2_policy_evict_first();  // V is read once per sample
            auto load_v = [&](int t, int s2) {  // V' tile: rows i, 64 columns u per box
                const int ti = t / p.tiles_u, tu = t % p.tiles_u;
                for (int q = 0; q < 2; q++)
                    tma_load_3d_hint(const_cast<__nv_bfloat16 *>(sV(s2)) + q * (kQTile * 64), &tmV, 0, 0,
                                     ti * p.kb64 + 2 * tu + q, &full[s2], vpol);
            };
            auto load_ab = [&](int t, int s2) {
                const int ti = t / p.tiles_u, tu = t % p.tiles_u;
                for (int q = 0; q < 2; q++) {
                    tma_load_2d(sA(s2) + q * boxBytes, &tmA, ti * kQTile + q * 64, 0, &full[s2]);
                    tma_load_2d(sB(s2) + q * boxBytes, &tmB, tu * kQTile + q * 64, 0, &full[s2]);
                }
            };
            int pre = 0;  // fresh stages: no empty wait
            for (int t = blockIdx.x; t < T && pre < p.stages; t += gridDim.x, pre++) {
                mbar_arrive_expect_tx(&full[pre], (uint32_t)stageBytes);
                load_v(t, pre);
            }
            griddep_wait();
            griddep_launch_dependents();
            for (int k = 0; k < pre; k++) {
                load_ab(blockIdx.x + k * gridDim.x, k);
                armed[k]++;
            }
            st = pre == p.stages ? 0 : pre;
            ph = pre == p.stages ? 1u : 0u;
            for (int t = blockIdx.x + pre * gridDim.x; t < T; t += gridDim.x) {
                if (!mbar_wait(&empty[st], ph ^ 1, p.err, kErrWaitEmpty, p.wait_limit)) break;
                mbar_arrive_expect_tx(&full[st], (uint32_t)stageBytes);
                load_ab(t, st);
                load_v(t, st);
                armed[st]++;
                if (++st == p.stages) {
                    st = 0;
                    ph ^= 1;
                }
            }
            if (*((volatile int *)p.err) != 0)
                for (int k = 0; k < p.stages; k++)
                    if (armed[k] > 0) mbar_wait_quiet(&full[k], (uint32_t)((armed[k] - 1) & 1));
        } else {
            griddep_wait();
            griddep_launch_dependents();
        }
    } else if (warp == 1) {
        griddep_wait();
        griddep_launch_dependents();
        if (lane == 0) {
            // both operands MN-major: a K16 step is 16 rows of 128 bytes; the second 64-wide box of M / N
            // is boxBytes further (leading byte offset), 8-row groups 1024 bytes apart
            const uint32_t idesc = idesc_bf16_f32(kQTile, kQTile) | kIdescAMnMajor | kIdescBMnMajor;
            int st = 0, acc = 0;
            uint32_t ph = 0, aph = 0;
            for (int t = blockIdx.x; t < T; t += gridDim.x) {
                if (!mbar_wait(&tempty[acc], aph ^ 1, p.err, kErrWaitTmemEmpty, p.wait_limit)) break;
                if (!mbar_wait(&full[st], ph, p.err, kErrWaitFull, p.wait_limit)) break;
                tc_fence_after();
                const uint32_t a0 = smem_u32(sA(st)), b0 = smem_u32(sB(st));
                for (int k16 = 0; k16 < p.npad / 16; k16++)
                    tc_mma_f16(tmem + (uint32_t)(acc * kQTile), smem_desc(a0 + k16 * 2048, boxBytes, 1024, 2),
                               smem_desc(b0 + k16 * 2048, boxBytes, 1024, 2), idesc, k16 > 0 ? 1u : 0u);
                tc_commit(&empty[st]);
                tc_commit(&tfull[acc]);
                if (++st == p.stages) {
                    st = 0;
                    ph ^= 1;
                }
                if (++acc == 2) {
                    acc = 0;
                    aph ^= 1;
                }
            }
            tc_commit(mdone);
            mbar_wait_quiet(mdone, 0);
        }
    } else {
        griddep_wait();
        griddep_launch_dependents();
        const int quarter = warp & 3;          // TMEM lanes this warp may read
        const int c0 = ((warp - 2) >> 2) * 32; // its 32 columns of the tile
        const int i = quarter * 32 + lane;     // this thread's row of the tile (its TMEM lane)
        // eps > 0 keeps the log finite in zero-padded rows and columns (V = 0 there, so they add 0)
        const float eps = fmaxf(p.eps, 1e-30f);
        double dlog = 0.0, ds = 0.0;
        int st = 0, acc = 0;
        uint32_t ph = 0, aph = 0;
        for (int t = blockIdx.x; t < T; t += gridDim.x) {
            if (!warp_wait(&tfull[acc], aph, p.err, kErrWaitTmemFull, p.wait_limit)) break;
            if (!warp_wait(&full[st], ph, p.err, kErrWaitFull, p.wait_limit)) break;  // the V tile of this stage
            tc_fence_after();
            const __nv_bfloat16 *v = sV(st);
            const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * kQTile + c0);
            float sv[32];
            {
                float a[16], b[16];
                tmem_ld16(taddr, a);
                tmem_ld16(taddr + 16, b);
                tmem_ld_wait();
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    sv[j] = a[j];
                    sv[16 + j] = b[j];
                }
            }
            // this row's 32 values of V: 4 chunks of 8 in the 128-byte swizzled row i of box c0 / 64
            const unsigned char *vrow =
                reinterpret_cast<const unsigned char *>(v + (c0 >> 6) * (kQTile * 64)) + i * 128;
            float plog[4] = {0.f, 0.f, 0.f, 0.f}, ps[4] = {0.f, 0.f, 0.f, 0.f};  // four independent sums each
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int chunk = (((c0 & 63) >> 3) + k) ^ (i & 7);
                const uint4 raw = *reinterpret_cast<const uint4 *>(vrow + chunk * 16);
                const __nv_bfloat162 *h2 = reinterpret_cast<const __nv_bfloat162 *>(&raw);
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const float2 vv = __bfloat1622float2(h2[e]);
                    const int j = 8 * k + 2 * e;
                    plog[e] = fmaf(vv.x, lg2_approx(sv[j] + eps), plog[e]);
                    plog[e] = fmaf(vv.y, lg2_approx(sv[j + 1] + eps), plog[e]);
                    ps[e] += sv[j];
                    ps[e] += sv[j + 1];
                }
            }
            dlog += (double)((plog[0] + plog[1]) + (plog[2] + plog[3]));
            ds += (double)((ps[0] + ps[1]) + (ps[2] + ps[3]));
            tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&tempty[acc]);
                mbar_arrive(&empty[st]);
            }
            if (++st == p.stages) {
                st = 0;
                ph ^= 1;
            }
            if (++acc == 2) {
                acc = 0;
                aph ^= 1;
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            dlog += __shfl_down_sync(0xffffffffu, dlog, off);
            ds += __shfl_down_sync(0xffffffffu, ds, off);
        }
        if (lane == 0) {
            red[warp - 2] = dlog;
            red[kQEpiWarps + warp - 2] = ds;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double l = 0.0, sm = 0.0;
        for (int w = 0; w < kQEpiWarps; w++) {
            l += red[w];
            sm += red[kQEpiWarps + w];
        }
        p.partial[blockIdx.x] = 0.30102999566398120 * l - sm;  // log10(x) = log2(x) log10(2)
        // publishes this partial; the last CTA's add also acquires every other CTA's
        reinterpret_cast<volatile int *>(red)[0] = atom_acq_rel_add(p.done, 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (warp == 0 && reinterpret_cast<volatile int *>(red)[0]) {
        // the last CTA: the partials summed in CTA order (lane-strided, then a fixed tree), so the
        // value does not depend on which CTA finished last
        double q = 0.0;
        for (int c = lane; c < (int)gridDim.x; c += 32) q += __ldcg(p.partial + c);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) q += __shfl_down_sync(0xffffffffu, q, off);
        if (lane == 0) {
            p.out[0] = (float)q;
            if (p.out_host) {
                p.out_host[0] = (float)q;
                __threadfence_system();
            }
            *p.done = 0;
        }
    }
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 2 * kQTile);
    }
}

// ------------------------------------------------------------------------
// conversions
// ------------------------------------------------------------------------
// V (n x m FP32 column-major) -> Vb and Vbt in the tiled layout (16 KB chunks of 128 rows x 64 K,
// zero beyond n and m): one 64 x 64 block of (i, u) per CTA through shared memory; each warp writes
// whole 128-byte chunk rows (32 threads x two BF16 values).  npr, mpr: n, m rounded up to 128.
// V may be host memory the device can read (the job's creation reads the caller's matrix once,
// over the host link, instead of copying it first); then Vcopy receives the FP32 device copy.
__global__ void __launch_bounds__(256) convert_v_kernel(const float *__restrict__ V, int n, int m, int npr, int mpr,
                                                        __nv_bfloat16 *__restrict__ Vb, __nv_bfloat16 *__restrict__ Vbt,
                                                        float *__restrict__ Vcopy) {
    __shared__ float tile[64][65];
    const int i0 = blockIdx.x * 64, u0 = blockIdx.y * 64;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;  // 8 warps
    const long long kb64i = npr / 64, kb64u = mpr / 64;
    const int i = i0 + 2 * lane;
    // rows u of the block (8 per warp): 64 values of i each, all loads issued before any store
    float a[8], b[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int u = u0 + w + 8 * q;
        a[q] = (u < m && i < n) ? V[(long long)u * n + i] : 0.f;
        b[q] = (u < m && i + 1 < n) ? V[(long long)u * n + i + 1] : 0.f;
    }
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int uu = w + 8 * q, u = u0 + uu;
        tile[uu][2 * lane] = a[q];
        tile[uu][2 * lane + 1] = b[q];
        __nv_bfloat16 *dst = Vb + (((long long)(u >> 7) * kb64i + (i0 >> 6)) * 128 + (u & 127)) * 64 + 2 * lane;
        *reinterpret_cast<__nv_bfloat162 *>(dst) = __floats2bfloat162_rn(a[q], b[q]);
        if (Vcopy && u < m) {
            if (i < n) Vcopy[(long long)u * n + i] = a[q];
            if (i + 1 < n) Vcopy[(long long)u * n + i + 1] = b[q];
        }
    }
    __syncthreads();
    // rows i of the block: 64 values of u each, one chunk row of Vbt
    for (int ii = w; ii < 64; ii += 8) {
        const int ir = i0 + ii;
        __nv_bfloat16 *dst = Vbt + (((long long)(ir >> 7) * kb64u + (u0 >> 6)) * 128 + (ir & 127)) * 64 + 2 * lane;
        *reinterpret_cast<__nv_bfloat162 *>(dst) = __floats2bfloat162_rn(tile[2 * lane][ii], tile[2 * lane + 1][ii]);
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
        // numerators: the tile's partial slots summed in slot order.  Rows lrow0 + c < 128 of a slot
        // (RP == npad) are in bounds for every c < kUpdCols, so the loads need no column guard (the
        // sums over the tile's padding rows are never stored).  The table lists a tile's slots
        // first, then -1: four slots' loads are issued together (an absent slot reads the first one
        // again and is not added); a branch around each slot's loads would serialise them.
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
            for (int q0 = 0; q0 < kSlotW; q0 += 4) {
                if (q0 > 0 && sl[q0] < 0) continue;
                float v[4][PER];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int sq = sl[q0 + q] >= 0 ? sl[q0 + q] : sl[0];
                    const float *base = p.P + ((size_t)sq * 128 + lrow0) * p.npad;
#pragma unroll
                    for (int j = 0; j < PER; j++) {
                        const int k = tid + j * kUpdThreads, c = k / RP, a = k % RP;
                        v[q][j] = base[c * p.npad + a];
                    }
                }
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (sl[q0 + q] >= 0) {
#pragma unroll
                        for (int j = 0; j < PER; j++) acc[j] += v[q][j];
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
// never materialising W H.  Per 128-row output tile and 128-wide K block:
//   MMA1  D1[128 x 128] = A1[128 x r] F[128 x r]^T     (S for the block, in TMEM)
//   epilogue warps: R = V / (D1 + eps) -> BF16, stored back into the same
//                   TMEM columns (two values per 32-bit column)
//   MMA2  D2[128 x r]  += R[128 x 128] F[128 x r]      (numerator, in TMEM;
//                   A read from TMEM, B = the same F tile read MN-major)
//   H-step: rows u; A1 = Hc (H, column-major BF16), F = Wr (W, row-major),
//           V tile from Vb;                  K = i (rows of V)
//   W-step: rows i; A1 = Wr, F = Hc, V tile from Vbt;  K = u
// One F tile serves both products, so a block moves 32 KB of V (HBM) and
// r*256 bytes of F (L2) into shared memory, and the tensor pipe gets 8 + 8
// instructions of N = 128 per block (r = 128), few enough for one issuing
// thread.  V and F have separate rings: a V stage is released as soon as the
// epilogue has read it, an F stage when MMA2 of its block completes.  TMEM
// holds nb S/R buffers of 128 columns and the numerator accumulator, so MMA1
// runs up to nb blocks ahead of the epilogue; the MMA thread polls its
// barriers and issues whichever product is ready (MMA2 first, which frees
// buffers).  Stream-K partition and partial slots as in the Euclidean GEMM;
// the epilogue warps also finish the column/row sums (the KL denominators)
// from the update kernel's partials.
// ========================================================================
struct KlParams {
    int tiles, kblocks, npad, max_seg, nbox;
    int kb64;        // 64-wide chunks of V per row tile along K (the tiled layout)
    int sv, sf, nb;  // V ring stages, F ring stages, S/R buffers in TMEM
    float eps;
    float *partials;
    int *err;
    long long wait_limit;
    const float *sum_partials;  // [count][npad] partial sums of the other factor
    float *sum_out;             // [npad]
    int sum_count;
    // fused update (X != null): after the stream every CTA updates its slice of the factor's rows,
    // [c*rows/G, (c+1)*rows/G), from its tiles' partial slots (as the separate update kernel does)
    float *X;                   // H (r x m, element (a, u) at u*r + a) or W (n x r, (i, a) at a*ldx + i)
    __nv_bfloat16 *Xb, *Xr;     // BF16 copies: (a, row) at a*ldb + row; (row, a) at row*ldr + a
    long long ldb, ldr, ldx;
    int is_w, rows, r, additive;
    const int *slot_ptr, *slot_list;  // each tile's slots in K order
    int *tile_cnt, *tile_rd;          // per tile: partial products out, readers done (the last resets)
    const int *tile_readers;          // per tile: how many CTAs read it
    int *sum_cnt;                     // [2]: CTAs whose denominator entries are out; CTAs done (last resets)
    float *sum_part_out;              // [grid][npad] sums of this CTA's new rows (the next kernel's denominators)
};

constexpr int kKlEpiWarps = 16;  // 4 per TMEM lane quarter, 32 columns of each block each
constexpr int kKlThreads = 64 + 32 * kKlEpiWarps;  // warp 0 TMA, warp 1 MMA, then the ratio epilogue

// Fused KL update (all 576 threads, after the stream; the rings' shared memory is free).  For each
// chunk of up to 128 of this CTA's rows: wait until the chunk's tiles have all their partial
// products (and, before the first, until every CTA has published its denominator entries), copy the
// chunk's rows of every slot into shared memory at once (cp.async), sum them in K order, apply
// X *= num / max(sum, eps) (nmf_kernels.cu:289,337), or X = max(0, X + X / max(sum, eps) (num - sum))
// for the additive rule (nmf_kernels_additive_divergence.cu:101-104), write X and its two BF16
// copies, and add the new rows to this CTA's sums, the next kernel's denominators.  The host checks
// that the staging fits (rows x slots per chunk).
template <int NP>
__device__ __forceinline__ void kl_fused_tail(const KlParams &p, float *smem, int *sflag) {
    constexpr int LD = NP + 1;  // sX[128][NP + 1]
    const int tid = threadIdx.x, c = blockIdx.x, G = gridDim.x;
    const int rows = p.rows, r = p.r;
    const long long x0 = (long long)c * rows / G, x1 = (long long)(c + 1) * rows / G;
    float *sX = smem;
    float *sSum = sX + 128 * LD, *sRaw = sSum + NP;
    float *sP = sRaw + NP;  // staged slot rows: [part][slot][row][NP]
    float colsum = 0.f;     // thread a < NP: this CTA's sum of the new X(., a)
    bool first = true;
    for (long long xb = x0; xb < x1; xb += 128) {
        const int nr = (int)min(128LL, x1 - xb);
        const int t0 = (int)(xb / kTileM), t1 = (int)((xb + nr - 1) / kTileM);  // t1 <= t0 + 1
        const int split = (int)min((long long)nr, (long long)(t0 + 1) * kTileM - xb);  // rows in t0
        // once past the waits, count this CTA as a reader of the chunk's tiles; the answers are used
        // at the end of the chunk, where the last reader of a tile resets its counters
        int rd0 = 0, rd1 = 0, last0 = -1, last1 = -1;
        if (tid == 0) {
            last0 = p.tile_readers[t0] - 1;
            if (t1 > t0) last1 = p.tile_readers[t1] - 1;
            bool ok = !first || flag_wait_ge(p.sum_cnt, G, p.err, kErrWaitTile, p.wait_limit);
            for (int t = t0; t <= t1 && ok; t++)
                ok = flag_wait_ge(p.tile_cnt + t, p.slot_ptr[t + 1] - p.slot_ptr[t], p.err, kErrWaitTile,
                                  p.wait_limit);
            if (ok) {
                rd0 = atomicAdd(p.tile_rd + t0, 1);
                if (t1 > t0) rd1 = atomicAdd(p.tile_rd + t1, 1);
            }
            sflag[0] = ok ? 1 : 0;
        }
        __syncthreads();        // thread 0's acquire loads and this barrier order the reads below
        if (!sflag[0]) return;  // uniform; the error word is set
        // stage: part k covers chunk rows [k ? split : 0, k ? nr : split) of tile t0 + k
        const int ns0 = p.slot_ptr[t0 + 1] - p.slot_ptr[t0];
        const int ns1 = t1 > t0 ? p.slot_ptr[t1 + 1] - p.slot_ptr[t1] : 0;
        const int n0 = split, n1 = nr - split;
        const int lr0 = (int)(xb - (long long)t0 * kTileM);  // first chunk row's row in tile t0
        float *sP1 = sP + (size_t)ns0 * n0 * NP;
        {
            const int q4 = NP / 4, per0 = ns0 * n0 * q4, total = per0 + ns1 * n1 * q4;
            for (int k = tid; k < total; k += kKlThreads) {
                int part = k >= per0, kk = part ? k - per0 : k;
                const int nrows = part ? n1 : n0;
                const int q = kk / (nrows * q4), rem = kk - q * nrows * q4;
                const int rho = rem / q4, a4 = rem - rho * q4;
                const int t = t0 + part, lr = part ? rho : lr0 + rho;
                const int slot = p.slot_list[p.slot_ptr[t] + q];
                const float *src = p.partials + ((size_t)slot * kTileM + lr) * NP + 4 * a4;
                float *dst = (part ? sP1 : sP) + ((size_t)q * nrows + rho) * NP + 4 * a4;
                cp_async16(dst, src, true);
            }
            cp_async_commit();
        }
        if (first) {
            for (int a = tid; a < NP; a += kKlThreads) {
                const float sraw = __ldcg(p.sum_out + a);
                sRaw[a] = sraw;
                sSum[a] = fmaxf(sraw, p.eps);
            }
            first = false;
        }
        cp_async_wait_all();
        __syncthreads();
        // numerators (slots in K order) and the update
        for (int e = tid; e < nr * NP; e += kKlThreads) {
            const int rho = e / NP, a = e - rho * NP;
            const int part = rho >= split, prow = part ? rho - split : rho;
            const int ns = part ? ns1 : ns0, nrows = part ? n1 : n0;
            const float *base = (part ? sP1 : sP) + (size_t)prow * NP + a;
            float num = 0.f;
            for (int q = 0; q < ns; q++) num += base[(size_t)q * nrows * NP];
            float xn = 0.f;
            if (a < r) {
                const long long grow = xb + rho;
                const long long xi = p.is_w ? (long long)a * p.ldx + grow : grow * r + a;
                const float x = p.X[xi];
                if (p.additive) {
                    xn = x + (x / sSum[a]) * (num - sRaw[a]);
                    xn = xn < 0.f ? 0.f : xn;
                } else {
                    xn = x * (num / sSum[a]);
                }
                p.X[xi] = xn;
            }
            sX[rho * LD + a] = xn;
        }
        __syncthreads();
        // the BF16 copies: Xb (a, row) rows fastest; Xr (row, a) a fastest, zero beyond r
        for (int e = tid; e < r * nr; e += kKlThreads) {
            const int a = e / nr, rho = e - a * nr;
            p.Xb[(long long)a * p.ldb + xb + rho] = __float2bfloat16_rn(sX[rho * LD + a]);
        }
        for (int e = tid; e < nr * NP; e += kKlThreads) {
            const int rho = e / NP, a = e - rho * NP;
            p.Xr[(xb + rho) * p.ldr + a] = __float2bfloat16_rn(sX[rho * LD + a]);
        }
        if (tid < NP)
            for (int rho = 0; rho < nr; rho++) colsum += sX[rho * LD + tid];
        if (tid == 0) {
            if (rd0 == last0) {
                p.tile_cnt[t0] = 0;
                p.tile_rd[t0] = 0;
            }
            if (t1 > t0 && rd1 == last1) {
                p.tile_cnt[t1] = 0;
                p.tile_rd[t1] = 0;
            }
        }
        __syncthreads();
    }
    if (tid < NP) p.sum_part_out[(size_t)c * NP + tid] = colsum;
    if (tid == 0) {
        if (atomicAdd(p.sum_cnt + 1, 1) == G - 1) {  // every CTA is past its waits: reset
            p.sum_cnt[1] = 0;
            atomicExch(p.sum_cnt, 0);
        }
    }
}

constexpr int kKlBlockK = 128;            // K columns per block
constexpr int kKlVBytes = kTileM * kKlBlockK * 2;  // 32 KB: two 64-column boxes
constexpr int kKlFBox = kKlBlockK * 128;  // 16 KB: 128 K-rows x 64 columns of the factor
constexpr int kKlMaxSV = 6, kKlMaxSF = 8, kKlMaxNB = 3;
constexpr int kKlBarBytes = 1024;  // barriers, the TMEM address, the denominator scratch

// The hardware's approximate reciprocal (rcp.approx.ftz.f32, about 1 ulp): the ratio is rounded to
// BF16 afterwards, so this is exact enough, and it is a single special-function operation.
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ uint32_t sw128(int row, int chunk) {
    return (uint32_t)(row * 128 + ((chunk ^ (row & 7)) << 4));
}

// barrier of the 16 KL epilogue warps that ORs a per-thread flag (the same answer in every thread)
__device__ __forceinline__ bool kl_epi_bar_or(bool v) {
    unsigned r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, 3, 512, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((unsigned)v)
        : "memory");
    return r != 0;
}

// one lane of the (fully active) warp, the same every call
__device__ __forceinline__ bool elect_one() {
    uint32_t pred = 0;
    asm volatile("{\n\t.reg .pred P;\n\telect.sync _|P, 0xffffffff;\n\tselp.b32 %0, 1, 0, P;\n\t}" : "=r"(pred));
    return pred != 0;
}

__device__ __forceinline__ void ring_next(int &i, uint32_t &ph, int n) {
    if (++i == n) {
        i = 0;
        ph ^= 1;
    }
}


// NK = npad / 16: the K16 steps of MMA1 (compile-time, so the MMA thread issues straight-line code)
template <int NK>
__global__ void __launch_bounds__(kKlThreads)
    tc_kl_gemm_kernel(const __grid_constant__ CUtensorMap tmV, const __grid_constant__ CUtensorMap tmA1,
                      const __grid_constant__ CUtensorMap tmF, KlParams p) {
    constexpr int NP = NK * 16;
    const uintptr_t base = (reinterpret_cast<uintptr_t>(tc_dyn_smem) + 1023) & ~uintptr_t(1023);
    const int fBytes = p.nbox * kKlFBox;
    unsigned char *sFr = reinterpret_cast<unsigned char *>(base);
    unsigned char *sVr = sFr + p.sf * fBytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(sVr + p.sv * kKlVBytes);
    uint64_t *vfull = bars, *vempty = vfull + kKlMaxSV;
    uint64_t *ffull = vempty + kKlMaxSV, *fempty = ffull + kKlMaxSF;
    uint64_t *d1full = fempty + kKlMaxSF, *d1empty = d1full + kKlMaxNB, *rfull = d1empty + kKlMaxNB;
    uint64_t *tfull = rfull + kKlMaxNB, *tempty = tfull + 1;
    uint64_t *mdone = tempty + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mdone + 1);
    float *red = reinterpret_cast<float *>(mdone + 2);  // [16] per-warp sums of the denominators

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long T = (long long)p.tiles * p.kblocks;
    const long long lo = (long long)blockIdx.x * T / gridDim.x;
    const long long hi = (long long)(blockIdx.x + 1) * T / gridDim.x;
    auto sF = [&](int st) { return sFr + st * fBytes; };
    auto sV = [&](int st) { return sVr + st * kKlVBytes; };
    auto seg_end = [&](long long b) { return min(hi, (b / p.kblocks + 1) * p.kblocks); };

    if (threadIdx.x == 0) {
        for (int s = 0; s < p.sv; s++) {
            mbar_init(&vfull[s], 1);
            mbar_init(&vempty[s], kKlEpiWarps);  // every epilogue warp reads its part of each V tile
        }
        for (int s = 0; s < p.sf; s++) {
            mbar_init(&ffull[s], 1);
            mbar_init(&fempty[s], 1);
        }
        for (int b = 0; b < p.nb; b++) {
            mbar_init(&d1full[b], 1);
            mbar_init(&d1empty[b], 1);
            mbar_init(&rfull[b], kKlEpiWarps);
        }
        mbar_init(tfull, 1);
        mbar_init(tempty, kKlEpiWarps);
        mbar_init(mdone, 1);
        fence_mbar_init();
        tma_prefetch_desc(&tmV);
        tma_prefetch_desc(&tmA1);
        tma_prefetch_desc(&tmF);
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // TMEM columns: the numerator accumulator [0, npad), A1 (the tile's factor rows, BF16 pairs)
    // [npad, npad + 64), then nb S/R buffers of 128
    const uint32_t tD2 = tmem, tA1 = tmem + (uint32_t)NP, tD1 = tmem + (uint32_t)(NP + 64);
    // the previous kernel's outputs (the factor copies, the denominators' partials) are read only
    // after griddepcontrol.wait; V is not one of them, so the producer requests the first V stages
    // before it waits

    if (warp == 0) {
        if (lane == 0) {
            const uint64_t vpol = l2_policy_evict_first();  // V is read once per launch
            int vi = 0, fi = 0, seg = 0;
            uint32_t vph = 0, fph = 0;
            // the last phase armed on each full barrier (bit set) and its parity, for the drain below
            uint32_t armed_v = 0, par_v = 0, armed_f = 0, par_f = 0;
            bool ok = true;
            const long long vpre = min((long long)p.sv, hi - lo);  // fresh V stages: no empty wait
            for (long long bb = lo; bb < lo + vpre; bb++) {
                const int t = (int)(bb / p.kblocks), c0 = t * p.kb64 + (int)(bb % p.kblocks) * 2;
                mbar_arrive_expect_tx(&vfull[vi], (uint32_t)kKlVBytes);
                tma_load_3d_hint(sV(vi), &tmV, 0, 0, c0, &vfull[vi], vpol);
                tma_load_3d_hint(sV(vi) + kKlVBytes / 2, &tmV, 0, 0, c0 + 1, &vfull[vi], vpol);
                armed_v |= 1u << vi;
                par_v = (par_v & ~(1u << vi)) | (vph << vi);
                ring_next(vi, vph, p.sv);
            }
            griddep_wait();
            griddep_launch_dependents();
            for (long long b = lo; b < hi && ok;) {
                const int t = (int)(b / p.kblocks);
                const long long e = seg_end(b);
                // the factor rows of this row tile (MMA1's A), once per segment, as an entry of the F
                // ring (same size: nbox boxes of 128 rows x 64 columns); the MMA thread copies it
                // into TMEM and frees the entry
                if (!mbar_wait_sleep(&fempty[fi], fph ^ 1, p.err, kErrWaitEmpty, p.wait_limit)) break;
                mbar_arrive_expect_tx(&ffull[fi], (uint32_t)fBytes);
                for (int q = 0; q < p.nbox; q++) tma_load_2d(sF(fi) + q * kKlFBox, &tmA1, q * 64, t * kTileM, &ffull[fi]);
                armed_f |= 1u << fi;
                par_f = (par_f & ~(1u << fi)) | (fph << fi);
                ring_next(fi, fph, p.sf);
                for (long long bb = b; bb < e; bb++) {
                    const int k0 = (int)(bb % p.kblocks) * kKlBlockK;
                    if (!mbar_wait_sleep(&fempty[fi], fph ^ 1, p.err, kErrWaitEmpty, p.wait_limit)) {
                        ok = false;
                        break;
                    }
                    mbar_arrive_expect_tx(&ffull[fi], (uint32_t)fBytes);
                    for (int q = 0; q < p.nbox; q++) tma_load_2d(sF(fi) + q * kKlFBox, &tmF, q * 64, k0, &ffull[fi]);
                    armed_f |= 1u << fi;
                    par_f = (par_f & ~(1u << fi)) | (fph << fi);
                    ring_next(fi, fph, p.sf);
                    if (bb < lo + vpre) continue;  // its V is already on the way
                    if (!mbar_wait_sleep(&vempty[vi], vph ^ 1, p.err, kErrWaitEmpty, p.wait_limit)) {
                        ok = false;
                        break;
                    }
                    mbar_arrive_expect_tx(&vfull[vi], (uint32_t)kKlVBytes);
                    const int c0 = t * p.kb64 + (int)(bb % p.kblocks) * 2;
                    tma_load_3d_hint(sV(vi), &tmV, 0, 0, c0, &vfull[vi], vpol);
                    tma_load_3d_hint(sV(vi) + kKlVBytes / 2, &tmV, 0, 0, c0 + 1, &vfull[vi], vpol);
                    armed_v |= 1u << vi;
                    par_v = (par_v & ~(1u << vi)) | (vph << vi);
                    ring_next(vi, vph, p.sv);
                }
                seg++;
                b = e;
            }
            // no copy of this CTA may still be landing when it exits (after an error the consumers
            // stop early): wait, bounded, for the last phase armed on every barrier
            for (int s = 0; s < p.sf; s++)
                if (armed_f >> s & 1) mbar_wait_quiet(&ffull[s], par_f >> s & 1);
            for (int s = 0; s < p.sv; s++)
                if (armed_v >> s & 1) mbar_wait_quiet(&vfull[s], par_v >> s & 1);
        } else {
            griddep_wait();
            griddep_launch_dependents();
        }
    } else if (warp == 1) {
        griddep_wait();
        griddep_launch_dependents();
        // The MMA warp issues in a fixed order: MMA1 of the first nb blocks, then for every block j
        // MMA2(j) once its R is in TMEM, then MMA1(j + nb) into the S/R buffer MMA2(j) read, once
        // that MMA2 has completed.  Each step waits on the one barrier it needs, so a product is
        // issued as soon as its inputs are there.  The whole warp runs the loop (waits are voted),
        // one elected lane issues the products and commits.
        const uint32_t id1 = idesc_bf16_f32(kTileM, kKlBlockK);
        const uint32_t id2 = idesc_bf16_f32(kTileM, NP) | kIdescBMnMajor;
        // descriptors of A1 and of F stage 0 (K-major for MMA1, MN-major for MMA2: the factor's
        // 64-column boxes are the MN chunks, 16 KB apart); a stage or a K step moves the start
        // address, which is the descriptor's low bits (address >> 4)
        const uint64_t fdk = smem_desc(smem_u32(sFr), 16, 1024, 2);
        const uint64_t fdm = smem_desc(smem_u32(sFr), kKlFBox, 1024, 2);
        const uint32_t fstep = (uint32_t)fBytes >> 4;
        const bool leader = elect_one();
        // blocks of this CTA counted from 0; a segment ends at a tile boundary
        const int nblk = (int)(hi - lo);
        auto seg_end_local = [&](int j) { return (int)(seg_end(lo + j) - lo); };
        // spin on the barrier: the MMA warp's reaction is on the critical chain, and a sleeping
        // try_wait resumed a few hundred ns after the phase completed; the error word and the time
        // limit are checked now and then
        auto wait = [&](uint64_t *bar, uint32_t parity, int bit) {
            long long t0 = 0;
            for (int spin = 1;; spin++) {
                if (__all_sync(0xffffffffu, mbar_test(bar, parity))) return true;
                if ((spin & 63) == 0) {
                    if (__any_sync(0xffffffffu, *((volatile int *)p.err) != 0)) return false;
                    const long long now = __shfl_sync(0xffffffffu, clock64(), 0);
                    if (t0 == 0) {
                        t0 = now;
                    } else if (now - t0 > p.wait_limit) {
                        if (leader) atomicOr(p.err, bit);
                        return false;
                    }
                }
            }
        };
        // MMA1 cursor: block j1, its F-ring entry and S/R buffer; need_a1: the next entry is the A1
        // of a new segment (each segment's entries are its A1, then one F per block)
        int j1 = 0, e1 = seg_end_local(0), f1 = 0, d1 = 0;
        uint32_t f1ph = 0, d1ph = 0;
        bool need_a1 = true;
        // MMA1 of block j1; at a segment start the segment's A1 is copied from its F-ring entry into
        // TMEM first (ordered after the previous segment's MMA1s, which read the old A1, and before
        // the new ones; the entry is freed when the copy has completed)
        auto mma1 = [&]() -> bool {
            if (need_a1) {
                if (!wait(&ffull[f1], f1ph, kErrWaitFull)) return false;
                if (leader) {
                    tc_fence_after();
                    const uint64_t ad = fdk + (uint64_t)(f1 * fstep);
#pragma unroll
                    for (int k16 = 0; k16 < NK; k16++) {
                        const int off = (k16 >> 2) * kKlFBox + (k16 & 3) * 32;
                        tc_cp_128x256b(tA1 + (uint32_t)(k16 * 8), ad + (uint64_t)(off >> 4));
                    }
                    tc_commit(&fempty[f1]);
                }
                __syncwarp();
                ring_next(f1, f1ph, p.sf);
                need_a1 = false;
            }
            // the block's F tile, and its S/R buffer free (MMA2 of the block nb earlier completed)
            if (!wait(&ffull[f1], f1ph, kErrWaitFull) || !wait(&d1empty[d1], d1ph ^ 1, kErrWaitTmemEmpty))
                return false;
            if (leader) {
                tc_fence_after();
                const uint64_t fb = fdk + (uint64_t)(f1 * fstep);
                const uint32_t dd = tD1 + (uint32_t)(d1 * kKlBlockK);
#pragma unroll
                for (int k16 = 0; k16 < NK; k16++) {
                    const int offf = (k16 >> 2) * kKlFBox + (k16 & 3) * 32;
                    tc_mma_f16_ts(dd, tA1 + (uint32_t)(k16 * 8), fb + (uint64_t)(offf >> 4), id1, k16 > 0 ? 1u : 0u);
                }
                tc_commit(&d1full[d1]);
            }
            __syncwarp();
            ring_next(f1, f1ph, p.sf);
            ring_next(d1, d1ph, p.nb);
            if (++j1 == e1) {
                need_a1 = true;
                if (j1 < nblk) e1 = seg_end_local(j1);
            }
            return true;
        };
        bool ok = true;
        for (int q = 0; q < p.nb && j1 < nblk && ok; q++) ok = mma1();
        // MMA2 cursor (starts past the first segment's A1 entry)
        int j2 = 0, e2 = seg_end_local(0), f2 = 0, d2 = 0, seg2 = 0;
        uint32_t f2ph = 0, d2ph = 0;
        ring_next(f2, f2ph, p.sf);
        bool first2 = true;
        while (ok && j2 < nblk) {
            if (!wait(&rfull[d2], d2ph, kErrWaitTmemFull)) break;
            // the accumulator of a new segment: the previous segment's numerator drained
            if (first2 && seg2 > 0 && !wait(tempty, (uint32_t)((seg2 - 1) & 1), kErrWaitTmemEmpty)) break;
            if (leader) {
                tc_fence_after();
                const uint64_t fb = fdm + (uint64_t)(f2 * fstep);
                const uint32_t rb = tD1 + (uint32_t)(d2 * kKlBlockK);
#pragma unroll
                for (int k = 0; k < kKlBlockK / 16; k++)  // R of part p at columns 32p .. 32p + 15
                    tc_mma_f16_ts(tD2, rb + (uint32_t)((k >> 1) * 32 + (k & 1) * 8), fb + (uint64_t)(k * 2048 >> 4),
                                  id2, (first2 && k == 0) ? 0u : 1u);
                tc_commit(&fempty[f2]);
                tc_commit(&d1empty[d2]);
                if (j2 + 1 == e2) tc_commit(tfull);
            }
            __syncwarp();
            first2 = false;
            ring_next(f2, f2ph, p.sf);
            ring_next(d2, d2ph, p.nb);
            if (++j2 == e2) {
                seg2++;
                first2 = true;
                if (j2 < nblk) {
                    e2 = seg_end_local(j2);
                    ring_next(f2, f2ph, p.sf);  // past the next segment's A1 entry
                }
            }
            if (j1 < nblk) ok = mma1();
        }
        if (leader) {
            tc_commit(mdone);
            mbar_wait_quiet(mdone, 0);
        }
        __syncwarp();
    } else {
        griddep_wait();
        griddep_launch_dependents();
        // finish the denominators (column / row sums of the other factor) from the partials: each of
        // this CTA's entries by all 512 epilogue threads (thread et takes partials et, et + 512, ...,
        // then a fixed tree over lanes and warps), so no warp starts the ratios much later than the rest
        if (p.sum_out) {
            const int et = threadIdx.x - 64;  // 0 .. 511
            const int E = p.npad;
            const int e0 = (int)((long long)blockIdx.x * E / gridDim.x), e1 = (int)((long long)(blockIdx.x + 1) * E / gridDim.x);
            for (int ei = e0; ei < e1; ei++) {
                float v[4] = {0.f, 0.f, 0.f, 0.f};
                int z = et;
                for (; z + 3 * 512 < p.sum_count; z += 4 * 512) {
#pragma unroll
                    for (int q = 0; q < 4; q++) v[q] += p.sum_partials[(size_t)(z + q * 512) * E + ei];
                }
#pragma unroll
                for (int q = 0; q < 3; q++)  // at most three left
                    if (z + q * 512 < p.sum_count) v[q] += p.sum_partials[(size_t)(z + q * 512) * E + ei];
                float sacc = (v[0] + v[1]) + (v[2] + v[3]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
                if (lane == 0) red[warp - 2] = sacc;
                asm volatile("bar.sync 3, 512;" ::: "memory");
                if (et == 0) {
                    float t = 0.f;
                    for (int w = 0; w < kKlEpiWarps; w++) t += red[w];
                    p.sum_out[ei] = t;
                }
                asm volatile("bar.sync 3, 512;" ::: "memory");
            }
        }
        if (p.X && threadIdx.x == 64)  // this CTA's denominator entries are out (the fused tails wait)
            red_release_add(p.sum_cnt, 1);
        const int quarter = warp & 3;     // TMEM lanes this warp may access
        const int part = (warp - 2) >> 2;  // which 32 of the block's 128 columns; also its share of the D2 drain
        const float eps_pos = fmaxf(p.eps, 1e-30f);
        const int row = quarter * 32 + lane;
        const uint32_t lane_off = (uint32_t)(quarter * 32) << 16;
        int vi = 0, di = 0, seg = 0;
        uint32_t vph = 0, dph = 0;
        for (long long b = lo; b < hi;) {
            const long long e = seg_end(b);
            bool ok = true;
            // every block by all 16 warps (a quarter of the rows and a quarter of the columns each):
            // the ratio's latency, on the MMA1 -> MMA2 -> F-release chain, stays short
            for (long long bb = b; bb < e; bb++) {
                if (!mbar_wait_sleep(&d1full[di], dph, p.err, kErrWaitTmemFull, p.wait_limit) ||
                    !mbar_wait_sleep(&vfull[vi], vph, p.err, kErrWaitFull, p.wait_limit)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t ta = tD1 + (uint32_t)(di * kKlBlockK + part * 32) + lane_off;
                float sv[32];
                {
                    float (&s0)[16] = *reinterpret_cast<float (*)[16]>(&sv[0]);
                    float (&s1)[16] = *reinterpret_cast<float (*)[16]>(&sv[16]);
                    tmem_ld16(ta, s0);
                    tmem_ld16(ta + 16, s1);
                }
                // this part's 32 columns: 64-column box part / 2, 16-byte chunks 4 (part & 1) ..
                const unsigned char *vt = sV(vi) + (part >> 1) * (kKlVBytes / 2);
                uint4 vraw[4];
#pragma unroll
                for (int cc = 0; cc < 4; cc++) vraw[cc] = *reinterpret_cast<const uint4 *>(vt + sw128(row, (part & 1) * 4 + cc));
                // the V stage is read (the arrive orders the loads before the producer's refill)
                __syncwarp();
                if (lane == 0) mbar_arrive(&vempty[vi]);
                tmem_ld_wait();
                uint32_t rr[16];
#pragma unroll
                for (int cc = 0; cc < 4; cc++) {
                    const __nv_bfloat162 *v2 = reinterpret_cast<const __nv_bfloat162 *>(&vraw[cc]);
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        // eps_pos > 0 keeps zero-padded entries (V = 0, S = 0) at 0: 1/eps_pos is
                        // finite for eps_pos >= 1e-30.
                        const float2 vf = __bfloat1622float2(v2[q]);
                        const float r0 = vf.x * rcp_approx(sv[cc * 8 + 2 * q] + eps_pos);
                        const float r1 = vf.y * rcp_approx(sv[cc * 8 + 2 * q + 1] + eps_pos);
                        const __nv_bfloat162 o = __floats2bfloat162_rn(r0, r1);
                        rr[cc * 4 + q] = *reinterpret_cast<const uint32_t *>(&o);
                    }
                }
                // R (packed pairs) over the first 16 of this warp's 32 S columns, already read
                tmem_st16(ta, rr);
                tmem_st_wait();
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&rfull[di]);
                ring_next(vi, vph, p.sv);
                ring_next(di, dph, p.nb);
            }
            // the 16 warps leave together (the drain below ends at a barrier of all of them)
            if (kl_epi_bar_or(!ok)) break;
            if (kl_epi_bar_or(!mbar_wait_sleep(tfull, (uint32_t)(seg & 1), p.err, kErrWaitTmemFull, p.wait_limit))) break;
            tc_fence_after();
            float *dst = p.partials + ((size_t)(blockIdx.x * p.max_seg + seg) * kTileM + row) * p.npad;
            for (int c = part * 16; c < NP; c += 64) {  // the four warps of a quarter take turns by 16 columns
                float v[16];
                tmem_ld16(tD2 + lane_off + (uint32_t)c, v);
                tmem_ld_wait();
                float4 *d4 = reinterpret_cast<float4 *>(dst + c);
                d4[0] = make_float4(v[0], v[1], v[2], v[3]);
                d4[1] = make_float4(v[4], v[5], v[6], v[7]);
                d4[2] = make_float4(v[8], v[9], v[10], v[11]);
                d4[3] = make_float4(v[12], v[13], v[14], v[15]);
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(tempty);
            if (p.X) {  // this segment's partial product is out: count it on its tile (the 16 warps'
                        // stores are ordered before the barrier, one release publishes them)
                asm volatile("bar.sync 3, 512;" ::: "memory");
                if (threadIdx.x == 64) red_release_add(&p.tile_cnt[b / p.kblocks], 1);
            }
            seg++;
            b = e;
        }
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 512);
    }
    if (p.X && __syncthreads_and(*((volatile int *)p.err) == 0))
        kl_fused_tail<NP>(p, reinterpret_cast<float *>(base), reinterpret_cast<int *>(red + 16));
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

// COLS columns of H (rows of W) per CTA: 8 for the H-step (its m is the smaller side: more CTAs),
// 16 for the W-step.  The old rows are staged in shared memory (W: read along its columns, H: along
// the rank), then the numerators are summed with the rank fastest, so the loads of the partial slots
// ([slot][row][npad]) are coalesced for both factors.
constexpr int kKlUpdColsH = 8, kKlUpdColsW = 16;
template <int RP, bool IS_W, int COLS>
__global__ void __launch_bounds__(kUpdThreads) tc_kl_update_kernel(KlUpdParams p) {
    constexpr int LDX = COLS + 1;  // odd: rank-fastest accesses of Xs[a][c] hit distinct banks
    constexpr int TOT = RP * COLS;  // 128 (r <= 16 in the H-step) up to 2048 elements
    constexpr int XL = (TOT + kUpdThreads - 1) / kUpdThreads;
    __shared__ float Xs[RP * LDX];
    __shared__ float sumS[RP], sumR[RP];
    const int tid = threadIdx.x;
    const int c0 = blockIdx.x * COLS;
    const int ncol = min(COLS, p.cols - c0);
    const int r = p.r;
    griddep_wait();
    griddep_launch_dependents();
#pragma unroll
    for (int j = 0; j < XL; j++) {  // the old rows, zero beyond r and beyond the last column
        const int k = tid + j * kUpdThreads;
        if (TOT % kUpdThreads != 0 && k >= TOT) break;
        if (IS_W) {
            const int a = k / COLS, c = k % COLS;
            Xs[a * LDX + c] = (a < r && c < ncol) ? p.X[(long long)a * p.ldx + c0 + c] : 0.f;
        } else {
            const int c = k / RP, a = k % RP;
            Xs[a * LDX + c] = (a < r && c < ncol) ? p.X[(long long)(c0 + c) * r + a] : 0.f;
        }
    }
    if (tid < RP) {
        const float sraw = p.update ? p.sums[tid] : 0.f;
        sumS[tid] = p.update ? fmaxf(sraw, p.eps) : 1.f;
        sumR[tid] = sraw;
    }
    float acc[XL];
#pragma unroll
    for (int j = 0; j < XL; j++) acc[j] = 0.f;
    if (p.update) {  // element (c, a) of thread-slot j: c = k / RP, a = k % RP (rank fastest)
        // Rows lrow0 + c < 128 of a slot (RP == npad): in bounds for c up to COLS - 1, so the loads
        // need no column guard (sums over the tile's padding rows are never stored).
        const int tile = c0 / 128, lrow0 = c0 % 128;
        int off[XL];
#pragma unroll
        for (int j = 0; j < XL; j++) {
            const int k = tid + j * kUpdThreads;
            off[j] = (k / RP) * p.npad + k % RP;
        }
        auto live = [&](int j) { return TOT % kUpdThreads == 0 || tid + j * kUpdThreads < TOT; };
        if (p.tile_slots) {
            // the table lists a tile's slots first, then -1: four slots' loads are issued together
            // (an absent slot reads the first one again and is not added), in slot order as added
            const int4 *ts = reinterpret_cast<const int4 *>(p.tile_slots + (size_t)tile * kSlotW);
            const int4 sa = ts[0], sb = ts[1];
            const int sl[kSlotW] = {sa.x, sa.y, sa.z, sa.w, sb.x, sb.y, sb.z, sb.w};
#pragma unroll
            for (int q0 = 0; q0 < kSlotW; q0 += 4) {
                if (q0 > 0 && sl[q0] < 0) continue;
                float v[4][XL];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int sq = sl[q0 + q] >= 0 ? sl[q0 + q] : sl[0];
                    const float *bs = p.P + ((size_t)sq * 128 + lrow0) * p.npad;
#pragma unroll
                    for (int j = 0; j < XL; j++) v[q][j] = live(j) ? bs[off[j]] : 0.f;
                }
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (sl[q0 + q] >= 0) {
#pragma unroll
                        for (int j = 0; j < XL; j++) acc[j] += v[q][j];
                    }
            }
        } else {
            for (int q = p.slot_ptr[tile]; q < p.slot_ptr[tile + 1]; q++) {
                const float *bs = p.P + ((size_t)p.slot_list[q] * 128 + lrow0) * p.npad;
#pragma unroll
                for (int j = 0; j < XL; j++)
                    if (live(j)) acc[j] += bs[off[j]];
            }
        }
    }
    __syncthreads();
    if (p.update) {
#pragma unroll
        for (int j = 0; j < XL; j++) {
            const int k = tid + j * kUpdThreads, c = k / RP, a = k % RP;
            if (a < r && c < ncol) {
                float x = Xs[a * LDX + c];
                if (p.additive) {
                    x = x + (x / sumS[a]) * (acc[j] - sumR[a]);
                    x = x < 0.f ? 0.f : x;
                } else {
                    x *= (acc[j] / sumS[a]);
                }
                Xs[a * LDX + c] = x;
            }
        }
    }
    __syncthreads();
    if (p.update) {
        for (int k = tid; k < RP * COLS; k += kUpdThreads) {  // X: along W's columns / H's rank
            if (IS_W) {
                const int a = k / COLS, c = k % COLS;
                if (a < r && c < ncol) p.X[(long long)a * p.ldx + c0 + c] = Xs[a * LDX + c];
            } else {
                const int c = k / RP, a = k % RP;
                if (a < r && c < ncol) p.X[(long long)(c0 + c) * r + a] = Xs[a * LDX + c];
            }
        }
        for (int k = tid; k < RP * COLS; k += kUpdThreads) {  // Xb: c fastest
            const int a = k / COLS, c = k % COLS;
            if (a < r && c < ncol) p.Xb[(long long)a * p.ldb + c0 + c] = __float2bfloat16_rn(Xs[a * LDX + c]);
        }
        for (int k = tid; k < RP * COLS; k += kUpdThreads) {  // Xr: a fastest
            const int c = k / RP, a = k % RP;
            if (c < ncol) p.Xr[(long long)(c0 + c) * p.ldr + a] = __float2bfloat16_rn(a < r ? Xs[a * LDX + c] : 0.f);
        }
    }
    if (tid < RP) {
        float sacc = 0.f;
        for (int c = 0; c < COLS; c++) sacc += Xs[tid * LDX + c];
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
    CUtensorMap tmQ;  // H-step with a folded quality sample: Hb, boxes of 64 columns u x npad rows
    gpunmf::SkParams p;
    int grid = 0;
    int smem = 0;
    int smem_qf = 0;  // shared memory of the variant with the quality warps
    int fnp = 0;  // fused update rank (kernel template argument), 0 = separate update kernel
    int *slot_ptr = nullptr, *slot_list = nullptr;
    int *tile_slots = nullptr;
    int *counters = nullptr;  // [tiles] arrivals, [tiles] readers done, [tiles] readers, [2] Gram assembly
    float *grams = nullptr;   // [grid][npad^2] per-CTA Gram partials of the factor this GEMM updates
};

struct KlGemm {
    CUtensorMap tmV, tmA1, tmF;
    gpunmf::KlParams p;
    int grid = 0, smem = 0;
    int *slot_ptr = nullptr, *slot_list = nullptr, *tile_slots = nullptr;
    // fused update: whether it fits, its counters and the per-CTA sums of the new rows
    bool fusable = false;
    int *counters = nullptr;   // [tiles] arrivals, [tiles] readers done, [tiles] readers, [2] sums
    float *row_sums = nullptr; // [grid][npad]
};

struct TcState {
    __nv_bfloat16 *Vb = nullptr, *Vbt = nullptr, *Wb = nullptr, *Hb = nullptr;
    // KL rule: second BF16 layouts (W row-major, H column-major), denominators and their partials
    __nv_bfloat16 *Wr = nullptr, *Hc = nullptr;
    long long ldr = 0;
    KlGemm kh, kw;
    float *S_w = nullptr, *S_h = nullptr, *SP_w = nullptr, *SP_h = nullptr;
    long long ldw = 0, ldh = 0;
    int npr = 0, mpr = 0;  // n and m rounded up to 128: the extents of the tiled Vb / Vbt
    int npad = 16;
    TcGemm gh, gw;  // H-step (W'V) and W-step (VH')
    float *P_h = nullptr, *P_w = nullptr;
    int *err = nullptr;
    float *G_w = nullptr, *G_h = nullptr;     // W'W and H H', npad x npad
    // quality on the tensor cores: maps of Wr (W row-major), Hc (H column-major) and Vb
    CUtensorMap tmQA, tmQB, tmQV;
    gpunmf::QParams qp;
    int qgrid = 0, qsmem = 0;
    float *GP_w = nullptr, *GP_h = nullptr;   // per-CTA Gram partials of the update kernels
    int gp_w_count = 0, gp_h_count = 0;
    bool qfold = false;        // the quality sample can ride on the H-step (fused Euclidean jobs)
    bool qfold_armed = false;  // the next H-step carries it
    int max_ctas = 0;                         // CTAs per launch: the SMs, or fewer (gpunmf_set_grid_limit)
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

// CTAs per launch of the jobs created from now on (0: one per SM)
static std::atomic<int> g_grid_limit{0};

// Tiled BF16 copy of V (Vb or Vbt): `chunks` 16 KB chunks of 128 rows x 64 K values, 128-byte rows;
// box {64, 128, 1} = one chunk, 128B swizzle.
static gpunmf_status make_map_tiled(CUtensorMap *m, const void *base, uint64_t chunks) {
    auto fn = encode_fn();
    if (!fn) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return GPUNMF_ERR_CUDA;
    }
    cuuint64_t dims[3] = {64, 128, chunks};
    cuuint64_t strides[2] = {128, 128 * 128};
    cuuint32_t box[3] = {64, 128, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled (tiled V) failed (%d)", (int)r);
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

static int smem_optin() {
    static int v = 0;
    if (!v) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || v <= 0)
            v = 227 * 1024;
    }
    return v;
}

static gpunmf_status setup_gemm(gpunmf_job *j, TcGemm &g, int rows, int K, int npad, float **partials, int *err,
                                int fnp = 0) {
    const int tiles = ceil_div(rows, kTileM);
    const int boxB = npad * kBlockK * 2;
    // the fused epilogue's areas take shared memory from the stage ring; the separate update kernel
    // needs room beside a GEMM CTA instead
    const int budget = fnp ? smem_optin() - fused_smem_bytes(fnp) - 64 : kSmemBudget;
    // two 64-wide boxes per stage when at least three such stages fit, else one
    const int bps = (budget - 1280) / (2 * (kStageABytes + boxB)) >= 3 ? 2 : 1;
    const int kblocks = ceil_div(K, kBlockK * bps);
    const long long T = (long long)tiles * kblocks;
    g.grid = (int)std::min<long long>(j->tc->max_ctas, T);
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
    int stages = std::min(kMaxStages, (budget - 1024 - 256) / stage_bytes);
    // the fused kernel: at most three stages (96 KB of V per SM in flight).  More than that does not
    // raise the stream's bandwidth, only the time every other load waits behind it in the memory
    // system: the prologue's Gram reads and the grid-wide counters.  Measured at 8192 x 8192, r = 64:
    // 2 / 3 / 4 stages -> 12.9k / 13.6k / 13.2k iterations/s.
    if (fnp) stages = std::min(stages, 3);
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
    g.p.wait_limit = kWaitLimitCycles;
    g.smem = 1024 + stages * stage_bytes + (2 * stages + 5) * 8 + 16 + (fnp ? 16 + fused_smem_bytes(fnp) : 0);
    // with the folded quality sample: two H-tile slots, eight more barriers, the warps' sums
    g.smem_qf = g.smem + 2 * 2 * npad * kBlockK * 2 + (4 + 2 * kQfSBufs) * 8 + 2 * kQfWarps * 8;
    g.fnp = fnp;
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
    g.p.slot_ptr = g.slot_ptr;
    g.p.slot_list = g.slot_list;
    if (fnp) {
        // per tile: arrivals, readers done, readers expected; the Gram assembly counters; per CTA
        // the Gram partial of its new rows
        const int G = g.grid;
        std::vector<int> readers(tiles, 0);
        for (int c = 0; c < G; c++) {
            const long long x0 = (long long)c * rows / G, x1 = (long long)(c + 1) * rows / G;
            for (long long xb = x0; xb < x1; xb += 64) {
                const long long xe = std::min(x1, xb + 64);
                for (long long t = xb / kTileM; t <= (xe - 1) / kTileM; t++) readers[t]++;
            }
        }
        const size_t nc = (size_t)3 * tiles + 2;
        e = job_dev_alloc(j, (void **)&g.counters, nc * sizeof(int));
        if (e == cudaSuccess) e = cudaMemsetAsync(g.counters, 0, nc * sizeof(int), j->stream);
        if (e == cudaSuccess) e = job_h2d(j, g.counters + 2 * tiles, readers.data(), tiles * sizeof(int));
        if (e == cudaSuccess)
            e = job_dev_alloc(j, (void **)&g.grams, (size_t)G * fnp * fnp * sizeof(float));
        if (e != cudaSuccess) {
            set_error("fused-update workspace allocation failed: %s", cudaGetErrorString(e));
            cudaGetLastError();
            return GPUNMF_ERR_NOMEM;
        }
        g.p.tile_cnt = g.counters;
        g.p.tile_rd = g.counters + tiles;
        g.p.tile_readers = g.counters + 2 * tiles;
        g.p.red_cnt = g.counters + 3 * tiles;
        g.p.gp = g.grams;
    }
    return GPUNMF_OK;
}

// Largest number of stream-K segments on one tile for this GEMM shape (the fused update reads at
// most kFusedSlots per tile); mirrors setup_gemm's schedule.
static int schedule_max_slots(int rows, int K, int npad, int fnp, int max_ctas) {
    const int tiles = ceil_div(rows, kTileM);
    const int boxB = npad * kBlockK * 2;
    const int budget = fnp ? smem_optin() - fused_smem_bytes(fnp) - 64 : kSmemBudget;
    const int bps = (budget - 1280) / (2 * (kStageABytes + boxB)) >= 3 ? 2 : 1;
    const int kblocks = ceil_div(K, kBlockK * bps);
    const int grid = (int)std::min<long long>(max_ctas, (long long)tiles * kblocks);
    std::vector<int> ptr, list;
    int max_seg = 1;
    schedule(tiles, kblocks, grid, &max_seg, ptr, list);
    int mx = 0;
    for (int t = 0; t < tiles; t++) mx = std::max(mx, ptr[t + 1] - ptr[t]);
    return mx;
}

// rank of the fused update for a Euclidean job (npad 32 or 64), else 0
static int fused_rank(int npad) { return (npad == 32 || npad == 64) ? npad : 0; }

static size_t fused_bytes(int rows, int npad) {
    const int np = fused_rank(npad);
    if (!np) return 0;
    const int tiles = ceil_div(rows, kTileM);
    return (size_t)(3 * tiles + 2) * sizeof(int) + (size_t)kNumSMsGB300 * np * np * sizeof(float);
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
            result = cudaFuncSetAttribute(tc_gemm_sk_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        if (result == cudaSuccess)
            result = cudaFuncSetAttribute(tc_gemm_sk_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        if (result == cudaSuccess)
            result = cudaFuncSetAttribute(tc_gemm_sk_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        if (result == cudaSuccess)
            result = cudaFuncSetAttribute(tc_gemm_sk_kernel<32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        if (result == cudaSuccess)
            result = cudaFuncSetAttribute(tc_gemm_sk_kernel<64, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
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

constexpr int kKlMaxRank = 128;

static cudaError_t set_kl_smem_once() {
    static std::once_flag once;
    static cudaError_t result = cudaSuccess;
    std::call_once(once, [] {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        result = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
#define KLATTR(NK)                                                                                     \
    if (result == cudaSuccess)                                                                         \
        result = cudaFuncSetAttribute(tc_kl_gemm_kernel<NK>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        KLATTR(1) KLATTR(2) KLATTR(3) KLATTR(4) KLATTR(5) KLATTR(6) KLATTR(7) KLATTR(8)
#undef KLATTR
    });
    return result;
}

// The stream of the last launch per device of a grid whose CTAs wait on one another (see
// launch_resident); a job that is torn down (its stream drained first) forgets its stream here.
struct LastFused {
    std::mutex mu;
    cudaStream_t stream = nullptr;
    bool used = false;
    cudaEvent_t ev = nullptr;
};
static LastFused g_last_fused[64];

static void forget_fused_stream(cudaStream_t s) {
    for (LastFused &L : g_last_fused) {
        std::lock_guard<std::mutex> lock(L.mu);
        if (L.used && L.stream == s) L.used = false;
    }
}

// Launch of a grid whose CTAs wait on one another (every wait bounded): the grid (at most one CTA
// per SM) must be resident at once.  On one stream that holds: the previous kernel's CTAs never wait
// on the next one.  Two such grids on different streams could each hold part of the SMs and wait for
// the rest, so:
//  - a launch being captured into a graph (the server's iteration chunks, replayed on many streams)
//    is cooperative, which makes the residency of its grid a launch condition;
//  - otherwise these launches of this process are serialised across streams (a launch on a stream
//    other than the last one's first waits for everything submitted to that stream), which keeps the
//    programmatic dependent launch that a cooperative launch forgoes (~6% per iteration).
// at[0] holds the programmatic-serialisation attribute on entry; launch() launches with cfg.
template <class Launch>
static cudaError_t launch_resident(cudaLaunchConfig_t &cfg, cudaLaunchAttribute *at, Launch launch) {
    const cudaStream_t s = cfg.stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(s, &cap);
    if (e != cudaSuccess) return e;
    if (cap != cudaStreamCaptureStatusNone) {
        at[0].id = cudaLaunchAttributeCooperative;
        at[0].val.cooperative = 1;
        cfg.numAttrs = 1;
        return launch();
    }
    int dev = 0;
    cudaGetDevice(&dev);
    LastFused &L = g_last_fused[dev & 63];
    std::lock_guard<std::mutex> lock(L.mu);
    cudaStreamCaptureStatus lcap = cudaStreamCaptureStatusNone;
    if (L.used && L.stream != s && cudaStreamIsCapturing(L.stream, &lcap) == cudaSuccess &&
        lcap == cudaStreamCaptureStatusNone) {  // (work being captured there is not running yet)
        if (!L.ev) {
            e = cudaEventCreateWithFlags(&L.ev, cudaEventDisableTiming);
            if (e != cudaSuccess) return e;
        }
        e = cudaEventRecord(L.ev, L.stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, L.ev, 0);
        if (e != cudaSuccess) return e;
    }
    L.stream = s;
    L.used = true;
    return launch();
}

static gpunmf_status setup_kl(gpunmf_job *j, KlGemm &g, int rows, int K, int npad, float **partials, int *err) {
    const int tiles = ceil_div(rows, kTileM);
    const int kblocks = ceil_div(K, kKlBlockK);
    const long long T = (long long)tiles * kblocks;
    g.grid = (int)std::min<long long>(j->tc->max_ctas, T);
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
    // shared memory: A1 (nbox 16 KB boxes), the F ring (nbox 16 KB boxes a stage), the V ring
    // (32 KB a stage), barriers.  An F stage is held from its load until MMA2 of its block
    // completes (load, MMA1, ratio, MMA2: the longest chain of the pipeline), a V stage only until
    // the ratio has read it, so F gets at least four stages and V the rest (at least two).
    const int nbox = (npad + 63) / 64;
    const int fbytes = nbox * kKlFBox;
    const int fixed = 1024 + kKlBarBytes;
    const int room = smem_optin() - fixed;
    const int sv = std::max(2, std::min(kKlMaxSV, (room - 4 * fbytes) / kKlVBytes));
    const int sf = std::min(kKlMaxSF, (room - sv * kKlVBytes) / fbytes);
    if (sf < 2 || fixed + sv * kKlVBytes + sf * fbytes > smem_optin()) {
        set_error("KL tensor-core kernel: rank too large for the shared-memory pipeline");
        return GPUNMF_ERR_UNSUPPORTED;
    }
    g.p.tiles = tiles;
    g.p.kblocks = kblocks;
    g.p.npad = npad;
    g.p.max_seg = max_seg;
    g.p.nbox = nbox;
    g.p.sv = sv;
    g.p.sf = sf;
    g.p.nb = std::min(kKlMaxNB, (512 - npad - 64) / kKlBlockK);  // S/R buffers beside the accumulator and A1
    g.p.eps = j->eps;
    g.p.err = err;
    g.p.wait_limit = kWaitLimitCycles;
    g.smem = fixed + sv * kKlVBytes + sf * fbytes;
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
    // the fused update's staging (shared memory of the rings, free after the stream): per chunk of up
    // to 128 rows, the chunk's rows of every slot of its one or two tiles, next to the new rows
    {
        const int G = g.grid;
        const size_t room = (size_t)sv * kKlVBytes + (size_t)sf * fbytes;
        const size_t fixed_tail = ((size_t)128 * (npad + 1) + 2 * npad) * sizeof(float);
        std::vector<int> readers(tiles, 0);
        bool fits = true;
        for (int c = 0; c < G && fits; c++) {
            const long long x0 = (long long)c * rows / G, x1 = (long long)(c + 1) * rows / G;
            for (long long xb = x0; xb < x1; xb += 128) {
                const long long nr = std::min(128LL, x1 - xb);
                const int t0 = (int)(xb / kTileM), t1 = (int)((xb + nr - 1) / kTileM);
                const long long split = std::min(nr, (long long)(t0 + 1) * kTileM - xb);
                const long long ns0 = ptr[t0 + 1] - ptr[t0], ns1 = t1 > t0 ? ptr[t1 + 1] - ptr[t1] : 0;
                const size_t staged = (size_t)(ns0 * split + ns1 * (nr - split)) * npad * sizeof(float);
                if (fixed_tail + staged > room) fits = false;
                for (int t = t0; t <= t1; t++) readers[t]++;
            }
        }
        if (fits) {
            const size_t nc = (size_t)3 * tiles + 2;
            e = job_dev_alloc(j, (void **)&g.counters, nc * sizeof(int));
            if (e == cudaSuccess) e = cudaMemsetAsync(g.counters, 0, nc * sizeof(int), j->stream);
            if (e == cudaSuccess) e = job_h2d(j, g.counters + 2 * tiles, readers.data(), tiles * sizeof(int));
            if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&g.row_sums, (size_t)G * npad * sizeof(float));
            if (e != cudaSuccess) {
                set_error("KL fused-update workspace allocation failed: %s", cudaGetErrorString(e));
                cudaGetLastError();
                return GPUNMF_ERR_NOMEM;
            }
            g.fusable = true;
        }
    }
    return GPUNMF_OK;
}

// Per-CTA sums over a factor's rows, in the row partition of the fused update with G CTAs
// (out[c][a] = sum over rows [c*rows/G, (c+1)*rows/G) of X(row, a), in row order; 0 for a >= r):
// the denominators' partials of the first kernel, before any fused update has left them.
__global__ void kl_row_sums_kernel(const float *__restrict__ X, int is_w, long long ldx, int rows, int r,
                                   int npad, float *__restrict__ out) {
    const int c = blockIdx.x, G = gridDim.x;
    const long long x0 = (long long)c * rows / G, x1 = (long long)(c + 1) * rows / G;
    for (int a = threadIdx.x; a < npad; a += blockDim.x) {
        float s = 0.f;
        if (a < r)
            for (long long x = x0; x < x1; x++) s += is_w ? X[(long long)a * ldx + x] : X[x * r + a];
        out[(size_t)c * npad + a] = s;
    }
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
    auto launch = [&]() -> cudaError_t {
        switch (g.p.npad / 16) {
#define KLCASE(NK) \
    case NK: return cudaLaunchKernelEx(&cfg, tc_kl_gemm_kernel<NK>, g.tmV, g.tmA1, g.tmF, g.p);
            KLCASE(1) KLCASE(2) KLCASE(3) KLCASE(4) KLCASE(5) KLCASE(6) KLCASE(7) KLCASE(8)
#undef KLCASE
        }
        return cudaErrorInvalidValue;
    };
    // with the update fused its CTAs wait on one another (tile arrivals, the denominators)
    return g.p.X ? launch_resident(cfg, at, launch) : launch();
}

static cudaError_t launch_kl_update(const KlUpdParams &u, int rp, bool is_w, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ceil_div(u.cols, is_w ? kKlUpdColsW : kKlUpdColsH));
    cfg.blockDim = dim3(kUpdThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    switch (rp) {
#define CASE(R)                                                                                  \
    case R:                                                                                      \
        return is_w ? cudaLaunchKernelEx(&cfg, tc_kl_update_kernel<R, true, kKlUpdColsW>, u)     \
                    : cudaLaunchKernelEx(&cfg, tc_kl_update_kernel<R, false, kKlUpdColsH>, u);
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

static gpunmf_status setup_quality(gpunmf_job *j);

static gpunmf_status tc_create_kl(gpunmf_job *j) {
    TcState *t = j->tc;
    const int n = j->n, m = j->m, r = j->r;
    t->ldr = t->npad;
    const int cw = ceil_div(n, kKlUpdColsW), ch = ceil_div(m, kKlUpdColsH);  // the update kernels' CTAs
    cudaError_t e = job_dev_alloc(j, (void **)&t->Vb, (size_t)t->npr * t->mpr * 2);
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->Vbt, (size_t)t->npr * t->mpr * 2);
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
    if (t->kh.fusable && t->kw.fusable) {
        // each half-step updates its factor in its own tail: the H-step's rows are the columns u of
        // H, the W-step's the rows i of W; each leaves per-CTA sums of its new rows, which the other
        // half-step's kernel finishes into its denominators
        auto fuse = [&](KlGemm &g, float *X, __nv_bfloat16 *Xb, long long ldb, __nv_bfloat16 *Xr, long long ldx,
                        int is_w, int rows, const KlGemm &other) {
            const int tiles = g.p.tiles;
            g.p.X = X; g.p.Xb = Xb; g.p.ldb = ldb; g.p.Xr = Xr; g.p.ldr = t->ldr; g.p.ldx = ldx;
            g.p.is_w = is_w; g.p.rows = rows; g.p.r = r; g.p.additive = rule_is_additive(j->rule) ? 1 : 0;
            g.p.slot_ptr = g.slot_ptr; g.p.slot_list = g.slot_list;
            g.p.tile_cnt = g.counters; g.p.tile_rd = g.counters + tiles; g.p.tile_readers = g.counters + 2 * tiles;
            g.p.sum_cnt = g.counters + 3 * tiles;
            g.p.sum_part_out = g.row_sums;
            g.p.sum_partials = other.row_sums;
            g.p.sum_count = other.grid;
        };
        fuse(t->kh, j->H, t->Hb, t->ldh, t->Hc, 0, 0, m, t->kw);
        fuse(t->kw, j->W, t->Wb, t->ldw, t->Wr, n, 1, n, t->kh);
    }
    // H-step: rows u; V tile from Vb, A1 = Hc rows u, F = Wr rows i
    st = make_map_tiled(&t->kh.tmV, t->Vb, (uint64_t)(t->mpr / 128) * (t->npr / 64));
    t->kh.p.kb64 = t->npr / 64;
    t->kw.p.kb64 = t->mpr / 64;
    if (st == GPUNMF_OK) st = make_map(&t->kh.tmA1, t->Hc, r, m, t->ldr, kTileM);
    if (st == GPUNMF_OK) st = make_map(&t->kh.tmF, t->Wr, r, n, t->ldr, kKlBlockK);
    // W-step: rows i; V tile from Vbt, A1 = Wr rows i, F = Hc rows u
    if (st == GPUNMF_OK) st = make_map_tiled(&t->kw.tmV, t->Vbt, (uint64_t)(t->npr / 128) * (t->mpr / 64));
    if (st == GPUNMF_OK) st = make_map(&t->kw.tmA1, t->Wr, r, n, t->ldr, kTileM);
    if (st == GPUNMF_OK) st = make_map(&t->kw.tmF, t->Hc, r, m, t->ldr, kKlBlockK);
    if (st != GPUNMF_OK) return st;
    GPUNMF_CUDA_TRY(set_kl_smem_once());
    return setup_quality(j);
}

// Quality on the tensor cores (npad <= 128): the maps, the launch shape and the shared memory.
static gpunmf_status setup_quality(gpunmf_job *j) {
    TcState *t = j->tc;
    if (t->npad > 128) return GPUNMF_OK;  // the FP32 quality kernel serves larger ranks
    const int n = j->n, m = j->m, r = j->r;
    QParams &q = t->qp;
    q.tiles_i = ceil_div(n, kQTile);
    q.tiles_u = ceil_div(m, kQTile);
    q.npad = t->npad;
    q.eps = j->eps;
    q.err = t->err;
    q.wait_limit = kWaitLimitCycles;
    q.out = j->d_quality;
    {
        cudaError_t e = job_dev_alloc(j, (void **)&q.done, sizeof(int));
        if (e == cudaSuccess) e = cudaMemsetAsync(q.done, 0, sizeof(int), j->stream);
        if (e != cudaSuccess) {
            set_error("quality counter: %s", cudaGetErrorString(e));
            cudaGetLastError();
            return GPUNMF_ERR_NOMEM;
        }
        // the pinned read-back word, where the device can write it directly (mapped host memory)
        void *dp = nullptr;
        if (cudaHostGetDevicePointer(&dp, j->h_quality(), 0) == cudaSuccess) q.out_host = static_cast<float *>(dp);
        cudaGetLastError();
    }
    const int stageBytes = 4 * t->npad * 128 + kQVBytes;
    q.stages = std::min(3, (smem_optin() - 1024 - 256) / stageBytes);
    t->qsmem = 1024 + q.stages * stageBytes + (2 * q.stages + 5) * 8 + 8 + 2 * kQEpiWarps * 8 + 16;
    t->qgrid = (int)std::min<long long>(t->max_ctas, (long long)q.tiles_i * q.tiles_u);
    if (q.stages < 2 || (size_t)t->qgrid > j->red_cap) return GPUNMF_OK;  // not worth it here
    // Wb: {i, a}, Hb: {u, a}; boxes of 64 (contiguous) x npad (K rows; rows past r read zeros)
    gpunmf_status st = make_map(&t->tmQA, t->Wb, n, r, t->ldw, t->npad);
    if (st == GPUNMF_OK) st = make_map(&t->tmQB, t->Hb, m, r, t->ldh, t->npad);
    // V': chunks of 128 rows i x 64 columns u
    if (st == GPUNMF_OK) st = make_map_tiled(&t->tmQV, t->Vbt, (uint64_t)(t->npr / 128) * (t->mpr / 64));
    q.kb64 = t->mpr / 64;
    if (st != GPUNMF_OK) return st;
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(tc_quality_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_optin());
    });
    if (attr != cudaSuccess) {
        set_error("cudaFuncSetAttribute (quality): %s", cudaGetErrorString(attr));
        return GPUNMF_ERR_CUDA;
    }
    q.partial = j->red;
    // fused Euclidean jobs with an H-step sample the quality inside it (the H-step streams the same V)
    TcGemm &g = t->gh;
    if (g.fnp && j->rule != GPUNMF_ADDITIVE_EUCLIDEAN_FIXED_H && g.p.bps == 2 && (size_t)g.grid <= j->red_cap &&
        g.smem_qf <= smem_optin()) {
        g.tmQ = t->tmQB;
        g.p.qeps = j->eps;
        g.p.qpartial = j->red;
        g.p.qdone = q.done;
        g.p.qout = j->d_quality;
        g.p.qout_host = q.out_host;
        t->qfold = true;
    }
    return GPUNMF_OK;
}

bool tc_quality_fold(gpunmf_job *j) {
    if (!j->tc || !j->tc->qfold) return false;
    j->tc->qfold_armed = true;
    return true;
}

bool tc_quality_ready(const gpunmf_job *j) { return j->tc && j->tc->qp.partial != nullptr; }
bool tc_quality_writes_host(const gpunmf_job *j) { return j->tc && j->tc->qp.out_host != nullptr; }

// The quality of the current factors into j->d_quality (float), as the FP32 path leaves it.
gpunmf_status tc_quality(gpunmf_job *j) {
    TcState *t = j->tc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(t->qgrid);
    cfg.blockDim = dim3(kQThreads);
    cfg.dynamicSmemBytes = t->qsmem;
    cfg.stream = j->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    GPUNMF_CUDA_TRY(cudaLaunchKernelEx(&cfg, tc_quality_kernel, t->tmQA, t->tmQB, t->tmQV, t->qp));
    j->launches += 1;
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
        size_t b = 2 * (2 * (size_t)((n + 127) / 128 * 128) * ((m + 127) / 128 * 128) + (size_t)ceil8(n) * r +
                        (size_t)ceil8(m) * r + (size_t)(n + m) * npad);
        b += gemm_partial_bytes(m, n, npad) + gemm_partial_bytes(n, m, npad);
        b += (size_t)npad * sizeof(float) * (2 + ceil_div(n, kKlUpdColsW) + ceil_div(m, kKlUpdColsH)) + 64;
        return b;
    }
    size_t b = 2 * (2 * (size_t)((n + 127) / 128 * 128) * ((m + 127) / 128 * 128) + (size_t)ceil8(n) * r +
                    (size_t)ceil8(m) * r);
    b += gemm_partial_bytes(m, n, npad) + gemm_partial_bytes(n, m, npad);
    b += (size_t)npad * npad * sizeof(float) * (2 + ceil_div(n, kUpdCols) + ceil_div(m, kUpdCols)) + 64;
    b += fused_bytes(m, npad) + fused_bytes(n, npad);
    return b;
}

gpunmf_status tc_create(gpunmf_job *j) {
    TcState *t = new (std::nothrow) TcState();
    if (!t) return GPUNMF_ERR_NOMEM;
    j->tc = t;
    const int n = j->n, m = j->m, r = j->r;
    t->npad = npad_of(r);
    {
        const int cap = g_grid_limit.load();
        t->max_ctas = std::min(num_sms(), cap > 0 ? cap : INT_MAX);
        if (j->cta_cap > 0) t->max_ctas = std::min(t->max_ctas, j->cta_cap);
    }
    t->npr = (n + 127) / 128 * 128;
    t->mpr = (m + 127) / 128 * 128;
    t->ldw = ceil8(n);
    t->ldh = ceil8(m);
    if (rule_is_kl(j->rule)) return tc_create_kl(j);
    cudaError_t e = job_dev_alloc(j, (void **)&t->Vb, (size_t)t->npr * t->mpr * 2);
    if (e == cudaSuccess) e = job_dev_alloc(j, (void **)&t->Vbt, (size_t)t->npr * t->mpr * 2);
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
    int fnp = fused_rank(t->npad);
    if (fnp && (schedule_max_slots(m, n, t->npad, fnp, t->max_ctas) > kFusedSlots ||
                schedule_max_slots(n, m, t->npad, fnp, t->max_ctas) > kFusedSlots))
        fnp = 0;
    gpunmf_status st = setup_gemm(j, t->gh, m, n, t->npad, &t->P_h, t->err, fnp);
    if (st == GPUNMF_OK) st = setup_gemm(j, t->gw, n, m, t->npad, &t->P_w, t->err, fnp);
    if (st != GPUNMF_OK) return st;
    if (fnp) {
        // each GEMM updates its factor itself and leaves per-CTA Gram partials of it; the other
        // GEMM assembles the complete Gram from them (W'W for the H-step, H H' for the W-step)
        auto fill = [&](SkParams &q, float *X, __nv_bfloat16 *Xb, long long ldb, int is_w, int rows,
                        const TcGemm &other, float *G_full) {
            q.X = X; q.Xb = Xb; q.ldb = ldb; q.is_w = is_w; q.rows_valid = rows; q.r = r;
            q.additive = rule_is_additive(j->rule) ? 1 : 0; q.eps = j->eps;
            q.gin_parts = other.grams; q.gin_count = other.grid; q.G_full = G_full;
            q.gram_out = nullptr;
        };
        fill(t->gh.p, j->H, t->Hb, t->ldh, 0, m, t->gw, t->G_w);   // H-step: den = W'W H
        fill(t->gw.p, j->W, t->Wb, t->ldw, 1, n, t->gh, t->G_h);   // W-step: den = W H H'
    } else {
        // the H-step GEMM finishes W'W from the W-step update's partials, and vice versa
        t->gh.p.gram_partials = t->GP_w;
        t->gh.p.gram_out = t->G_w;
        t->gh.p.gram_count = t->gp_w_count;
        t->gh.p.gram_entries = (int)rp2;
        t->gw.p.gram_partials = t->GP_h;
        t->gw.p.gram_out = t->G_h;
        t->gw.p.gram_count = t->gp_h_count;
        t->gw.p.gram_entries = (int)rp2;
    }
    // H-step: rows = u (columns of V): A = Vb (dim0 i over n, dim1 u over m); B = Wb (dim0 i, dim1 a)
    st = make_map_tiled(&t->gh.tmA, t->Vb, (uint64_t)(t->mpr / 128) * (t->npr / 64));
    t->gh.p.kb64 = t->npr / 64;
    t->gw.p.kb64 = t->mpr / 64;
    if (st == GPUNMF_OK) st = make_map(&t->gh.tmB, t->Wb, n, r, t->ldw, t->npad);
    // W-step: rows = i: A = Vbt (dim0 u over m, dim1 i over n); B = Hb (dim0 u, dim1 a)
    if (st == GPUNMF_OK) st = make_map_tiled(&t->gw.tmA, t->Vbt, (uint64_t)(t->npr / 128) * (t->mpr / 64));
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
    return setup_quality(j);
}

gpunmf_status tc_prepare(gpunmf_job *j, const float *v_src) {
    TcState *t = j->tc;
    cudaStream_t s = j->stream;
    // from the job's V, or straight from the caller's matrix (which also fills the job's V)
    convert_v_kernel<<<dim3(t->npr / 64, t->mpr / 64), 256, 0, s>>>(v_src ? v_src : j->V, j->n, j->m, t->npr, t->mpr,
                                                                    t->Vb, t->Vbt, v_src ? j->V : nullptr);
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
        // column sums of the initial W, finished by the first H-step kernel: in the fused W-step's row
        // partition where the updates are fused, else as the update kernel leaves them
        if (t->kh.p.X) {
            kl_row_sums_kernel<<<t->kw.grid, 128, 0, s>>>(j->W, 1, j->n, j->n, j->r, t->npad, t->kw.row_sums);
            GPUNMF_CUDA_TRY(cudaGetLastError());
        } else {
            GPUNMF_CUDA_TRY(launch_kl_update(kl_params_w(j, 0), t->npad, true, s));
        }
        return GPUNMF_OK;
    }
    if (t->gh.fnp) {
        // the Gram partials of the initial W, where the W-step would leave them, for the first
        // H-step (and of the fixed H, where the H-step would leave them, for a rule without an
        // H step), over the same row partitions
        switch (t->gh.fnp) {
#define GP(NP)                                                                                          \
    case NP:                                                                                            \
        gram_partials_kernel<NP><<<t->gw.grid, 64, 0, s>>>(j->W, 1, j->n, j->r, t->gw.grams);          \
        GPUNMF_CUDA_TRY(cudaGetLastError());                                                            \
        if (j->rule == GPUNMF_ADDITIVE_EUCLIDEAN_FIXED_H) {                                             \
            gram_partials_kernel<NP><<<t->gh.grid, 64, 0, s>>>(j->H, 0, j->m, j->r, t->gh.grams);      \
            GPUNMF_CUDA_TRY(cudaGetLastError());                                                        \
        }                                                                                               \
        break;
            GP(32) GP(64)
#undef GP
        }
        return GPUNMF_OK;
    }
    // Gram partials of the initial W, finished by the first H-step GEMM
    GPUNMF_CUDA_TRY(launch_update(update_params_w(j, 0), t->npad, true, s));
    // a rule without an H step: the Gram partials of the (fixed) H, finished by every W-step GEMM
    if (j->rule == GPUNMF_ADDITIVE_EUCLIDEAN_FIXED_H)
        GPUNMF_CUDA_TRY(launch_update(update_params_h(j, 0), t->npad, false, s));
    return GPUNMF_OK;
}

static cudaError_t launch_gemm_cfg(TcGemm &g, cudaLaunchConfig_t &cfg, bool qf) {
    // (kernels without quality warps never read the third map)
    if (qf) {
        if (g.fnp == 32) return cudaLaunchKernelEx(&cfg, tc_gemm_sk_kernel<32, true>, g.tmA, g.tmB, g.tmQ, g.p);
        return cudaLaunchKernelEx(&cfg, tc_gemm_sk_kernel<64, true>, g.tmA, g.tmB, g.tmQ, g.p);
    }
    switch (g.fnp) {
        case 32: return cudaLaunchKernelEx(&cfg, tc_gemm_sk_kernel<32>, g.tmA, g.tmB, g.tmB, g.p);
        case 64: return cudaLaunchKernelEx(&cfg, tc_gemm_sk_kernel<64>, g.tmA, g.tmB, g.tmB, g.p);
        default: return cudaLaunchKernelEx(&cfg, tc_gemm_sk_kernel<0>, g.tmA, g.tmB, g.tmB, g.p);
    }
}

static cudaError_t launch_gemm(TcGemm &g, cudaStream_t s, bool qf = false) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(g.grid);
    cfg.blockDim = dim3(gemm_threads(g.fnp, qf));
    cfg.dynamicSmemBytes = qf ? g.smem_qf : g.smem;
    cfg.stream = s;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (!g.fnp) return launch_gemm_cfg(g, cfg, false);
    return launch_resident(cfg, at, [&] { return launch_gemm_cfg(g, cfg, qf); });
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
        // (one launch per half-step where the update is fused into the product kernel's tail)
        const bool fused = t->kh.p.X != nullptr;
        mark_begin(j);
        GPUNMF_CUDA_TRY(launch_kl_gemm(t->kh, s));
        mark_end(j);
        if (!fused) GPUNMF_CUDA_TRY(launch_kl_update(kl_params_h(j, 1), t->npad, false, s));
        j->launches += fused ? 1 : 2;
        if (!updateW) return GPUNMF_OK;
        // W <- W .* [(V ./ (WH + eps)) H'] ./ max(rowsum H, eps) with the new H
        mark_begin(j);
        GPUNMF_CUDA_TRY(launch_kl_gemm(t->kw, s));
        mark_end(j);
        if (!fused) GPUNMF_CUDA_TRY(launch_kl_update(kl_params_w(j, 1), t->npad, true, s));
        j->launches += fused ? 1 : 2;
        return GPUNMF_OK;
    }
    if (t->gh.fnp) {
        // one launch per half-step: the GEMM's last arrivals update the factor and its Gram
        if (j->rule != GPUNMF_ADDITIVE_EUCLIDEAN_FIXED_H) {
            const bool qf = t->qfold_armed;  // this H-step also samples the quality
            t->qfold_armed = false;
            mark_begin(j);
            GPUNMF_CUDA_TRY(launch_gemm(t->gh, s, qf));
            mark_end(j);
            j->launches += 1;
            if (qf) {
                if (!tc_quality_writes_host(j))
                    GPUNMF_CUDA_TRY(cudaMemcpyAsync(j->h_quality(), j->d_quality, sizeof(float), cudaMemcpyDeviceToHost, s));
                GPUNMF_CUDA_TRY(cudaEventRecord(j->qev, s));
                j->q_pending = true;
            }
        }
        if (!updateW) return GPUNMF_OK;
        mark_begin(j);
        GPUNMF_CUDA_TRY(launch_gemm(t->gw, s));
        mark_end(j);
        j->launches += 1;
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
    int e = 0;  // read in the job's stream order (its memory may be stream-ordered)
    GPUNMF_CUDA_TRY(cudaMemcpyAsync(&e, j->tc->err, sizeof(int), cudaMemcpyDeviceToHost, j->stream));
    GPUNMF_CUDA_TRY(cudaStreamSynchronize(j->stream));
    if (e != 0) {
        set_error("tensor-core kernel gave up waiting (error bits 0x%x)", e);
        return GPUNMF_ERR_TIMEOUT;
    }
    return GPUNMF_OK;
}

void tc_set_wait_limit(gpunmf_job *j, long long cycles) {
    TcState *t = j->tc;
    if (!t) return;
    const long long c = cycles > 0 ? cycles : kWaitLimitCycles;
    t->gh.p.wait_limit = t->gw.p.wait_limit = c;
    t->kh.p.wait_limit = t->kw.p.wait_limit = c;
    t->qp.wait_limit = c;
}

// Host-side fault injection: the arrival counter of the first row tile of the next H-step (the
// W-step where the rule has no H step) starts at -1 instead of 0, so after every partial product of
// that tile has arrived it stands one below the count the fused update waits for.  The wait runs
// out (bounded), the kernel sets the error word, the grid returns, and the host reports
// GPUNMF_ERR_TIMEOUT.  Only jobs whose updates are fused into the product kernels have the counter.
gpunmf_status tc_inject_missing_arrival(gpunmf_job *j) {
    TcState *t = j->tc;
    int *cnt = nullptr;
    if (t && rule_is_kl(j->rule)) {
        if (t->kh.p.X) cnt = t->kh.counters;
    } else if (t && t->gh.fnp) {
        cnt = j->rule == GPUNMF_ADDITIVE_EUCLIDEAN_FIXED_H ? t->gw.counters : t->gh.counters;
    }
    if (!cnt) {
        set_error("this job has no fused update (no tile arrival counters)");
        return GPUNMF_ERR_UNSUPPORTED;
    }
    GPUNMF_CUDA_TRY(cudaMemsetAsync(cnt, 0xFF, sizeof(int), j->stream));  // tile 0's count = -1
    return GPUNMF_OK;
}

void tc_set_grid_limit(int ctas) { g_grid_limit.store(ctas > 0 ? ctas : 0); }

void tc_destroy(gpunmf_job *j) {
    TcState *t = j->tc;
    if (!t) return;
    forget_fused_stream(j->stream);
    void *ptrs[] = {t->Vb, t->Vbt, t->Wb, t->Hb, t->P_h, t->P_w, t->err, t->G_h, t->G_w, t->GP_h, t->GP_w,
                    t->gh.slot_ptr, t->gh.slot_list, t->gw.slot_ptr, t->gw.slot_list,
                    t->gh.tile_slots, t->gw.tile_slots, t->Wr, t->Hc, t->S_w, t->S_h, t->SP_w, t->SP_h,
                    t->kh.slot_ptr, t->kh.slot_list, t->kh.tile_slots, t->kw.slot_ptr, t->kw.slot_list,
                    t->kh.counters, t->kh.row_sums, t->kw.counters, t->kw.row_sums,
                    t->kw.tile_slots, t->gh.counters, t->gh.grams, t->gw.counters, t->gw.grams};
    for (void *p : ptrs) job_dev_free(j, p);
    delete t;
    j->tc = nullptr;
}

}  // namespace gpunmf
