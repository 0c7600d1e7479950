// NMF job engine: the C ABI of include/gpunmf.h.
//
// A job owns device copies of V, W and H plus every workspace its rule
// needs, all allocated at creation (nothing is allocated per iteration).
// One iteration follows GPUMLib's order exactly:
//   Euclidean (src/algorithms/nmf/nmf_multiplicative_euclidian.cpp:29-67)
//     quality(W,H); H <- H .* (W'V) ./ (W'W H + eps); [W <- W .* (V H') ./ (W H H' + eps)]
//   KL (src/algorithms/nmf/nmf_multiplicative_divergence.cpp:29-50)
//     WH = W H; quality(WH); H <- H .* [W' (V./(WH+eps))] ./ max(colsum W, eps);
//     [WH = W H; W <- W .* [(V./(WH+eps)) H'] ./ max(rowsum H, eps)]
//   additive Euclidean (src/algorithms/nmf/nmf_additive_euclidian.cpp:29-57)
//     quality(W,H); H <- max(0, H + (H ./ W'W H) .* (W'V - W'W H));
//     [W <- max(0, W + (W ./ W H H') .* (V H' - W H H'))]
//     (the FIXED_H variant skips the H step, as the reference's GPU class does)
//   additive KL (src/algorithms/nmf/nmf_additive_divergence.cpp:29-51)
//     WH = W H; quality(WH); H <- max(0, H + (H ./ max(colsum W, eps)) .* W' (V./(WH+eps) - 1));
//     [WH = W H; W <- max(0, W + (W ./ max(rowsum H, eps)) .* (V./(WH+eps) - 1) H')]
// with the product arithmetic chosen per job: FP32 CUDA cores (the drop-in
// path) or BF16 tensor cores (tc_kernels.cu).
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <new>
#include <vector>

#include "common.cuh"
#include "engine.h"
#include "kernels.h"

namespace gpunmf {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

#define TRY_STATUS(expr)                          \
    do {                                          \
        gpunmf_status _s = (expr);                \
        if (_s != GPUNMF_OK) return _s;           \
    } while (0)

static gpunmf_status check_device() {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        set_error("no CUDA device available (%s)", e == cudaSuccess ? "count 0" : cudaGetErrorString(e));
        return GPUNMF_ERR_NO_DEVICE;
    }
    int dev = 0, major = 0, minor = 0;
    GPUNMF_CUDA_TRY(cudaGetDevice(&dev));
    GPUNMF_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    GPUNMF_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (major != 10 || minor != 3) {
        set_error("device %d is sm_%d%d; this library is built for sm_103a (GB300) only", dev, major, minor);
        return GPUNMF_ERR_NO_DEVICE;
    }
    return GPUNMF_OK;
}

// The library's memory pool of a device (created once): freed blocks stay in it (release threshold
// at its maximum) and are reused by later jobs; the default pool is left as the application set it.
static cudaMemPool_t library_pool(int dev) {
    static std::mutex mu;
    static cudaMemPool_t pools[64] = {};
    static bool tried[64] = {};
    std::lock_guard<std::mutex> lock(mu);
    const int k = dev & 63;
    if (!tried[k]) {
        tried[k] = true;
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        if (cudaMemPoolCreate(&pool, &props) == cudaSuccess) {
            unsigned long long thr = ~0ULL;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
            pools[k] = pool;
        } else {
            cudaGetLastError();  // no pool: plain allocations
        }
    }
    return pools[k];
}

static bool stream_ordered(const gpunmf_job *j) { return j->pool || j->async_alloc; }

cudaError_t job_dev_alloc(gpunmf_job *j, void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return cudaSuccess;
    if (j->pool) return cudaMallocFromPoolAsync(p, bytes, j->pool, j->stream);
    return j->async_alloc ? cudaMallocAsync(p, bytes, j->stream) : cudaMalloc(p, bytes);
}

void job_dev_free(gpunmf_job *j, void *p) {
    if (!p) return;
    if (stream_ordered(j))
        cudaFreeAsync(p, j->stream);
    else
        cudaFree(p);
}

cudaError_t job_h2d(gpunmf_job *j, void *dst, const void *src, size_t bytes) {
    if (bytes == 0) return cudaSuccess;
    // from pageable memory the call returns once the source is staged, so the caller may free it
    return stream_ordered(j) ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, j->stream)
                             : cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
}

template <class T>
static gpunmf_status dalloc(gpunmf_job *j, T **p, size_t count) {
    *p = nullptr;
    if (count == 0) return GPUNMF_OK;
    cudaError_t e = job_dev_alloc(j, (void **)p, count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        set_error("device allocation of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
        cudaGetLastError();
        return GPUNMF_ERR_NOMEM;
    }
    return GPUNMF_OK;
}

// ------------------------------------------------------------------------
// workspace sizing (shared by create and footprint)
// ------------------------------------------------------------------------
struct Sizes {
    int s_h, s_w, s_g;  // split-K slices: H-step product, W-step product, Gram products
    size_t p_h, p_w, p_g, d_h, d_w, wh, red;
};

static Sizes compute_sizes(int rule, int n, int m, int r, int precision) {
    Sizes z{};
    z.s_h = gemm_f32_splits(r, m, n);
    z.s_w = gemm_f32_splits(n, r, m);
    int sg1 = gemm_f32_splits(r, r, n), sg2 = gemm_f32_splits(r, r, m);
    z.s_g = sg1 > sg2 ? sg1 : sg2;
    z.p_h = (size_t)z.s_h * r * m;
    z.p_w = (size_t)z.s_w * n * r;
    const bool kl = rule_is_kl(rule);
    z.p_g = !kl ? (size_t)z.s_g * r * r : 0;
    z.d_h = !kl ? (size_t)r * m : 0;
    z.d_w = !kl ? (size_t)n * r : 0;
    z.wh = kl ? (size_t)n * m : 0;
    size_t red = 2 * (size_t)wh_reduce_ctas(n, m);
    size_t red2 = (size_t)quality_ew_ctas((long long)n * m);
    z.red = red > red2 ? red : red2;
    if (precision == GPUNMF_BF16) tc_add_sizes(rule, n, m, r, &z.red);
    return z;
}

size_t job_footprint(int rule, int n, int m, int r, int precision) {
    Sizes z = compute_sizes(rule, n, m, r, precision);
    size_t floats = (size_t)n * m + (size_t)n * r + (size_t)r * m + z.p_h + z.p_w + z.p_g + z.d_h + z.d_w +
                    z.wh + (size_t)r * r + (size_t)r + 8;
    size_t bytes = floats * sizeof(float) + z.red * sizeof(double) + 64;
    if (precision == GPUNMF_BF16) bytes += tc_footprint(rule, n, m, r);
    return bytes;
}

// ------------------------------------------------------------------------
// job lifetime
// ------------------------------------------------------------------------
static void job_free(gpunmf_job *j) {
    if (!j) return;
    if (j->tc) tc_destroy(j);
    float *fl[] = {j->V, j->W, j->H, j->P_h, j->P_w, j->P_g, j->G, j->D_h, j->D_w, j->WH, j->sums, j->d_quality};
    for (float *p : fl) job_dev_free(j, p);
    job_dev_free(j, j->red);
    job_dev_free(j, j->d_scalar);
    if (j->h_pinned && !j->external_pinned) cudaFreeHost(j->h_pinned);
    if (j->qev) cudaEventDestroy(j->qev);
    for (cudaEvent_t e : j->tev) cudaEventDestroy(e);
    if (j->own_stream && j->stream) cudaStreamDestroy(j->stream);
    delete j;
}

static gpunmf_status job_alloc(int rule, int n, int m, int r, float eps, int precision, void *stream,
                               gpunmf_job **out, unsigned char *pinned64 = nullptr, bool async_alloc = false,
                               int cta_cap = 0) {
    *out = nullptr;
    if (!rule_valid(rule)) {
        set_error("unknown rule %d", rule);
        return GPUNMF_ERR_INVALID;
    }
    if (precision != GPUNMF_FP32 && precision != GPUNMF_BF16) {
        set_error("unknown precision %d", precision);
        return GPUNMF_ERR_INVALID;
    }
    if (n <= 0 || m <= 0 || r <= 0) {
        set_error("invalid shape n=%d m=%d r=%d", n, m, r);
        return GPUNMF_ERR_INVALID;
    }
    if (!(eps >= 0.0f)) {
        set_error("eps must be >= 0");
        return GPUNMF_ERR_INVALID;
    }
    if ((long long)n * m > (1LL << 40)) {
        set_error("matrix too large");
        return GPUNMF_ERR_INVALID;
    }
    TRY_STATUS(check_device());
    if (precision == GPUNMF_BF16) {
        gpunmf_status st = tc_supported(rule, n, m, r);
        if (st != GPUNMF_OK) return st;
    }
    gpunmf_job *j = new (std::nothrow) gpunmf_job();
    if (!j) {
        set_error("host allocation failed");
        return GPUNMF_ERR_NOMEM;
    }
    j->cta_cap = cta_cap > 0 ? cta_cap : 0;
    j->rule = rule; j->n = n; j->m = m; j->r = r; j->eps = eps; j->precision = precision;
    j->async_alloc = async_alloc && stream != nullptr;
    if (stream) {
        j->stream = (cudaStream_t)stream;
        j->own_stream = false;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&j->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            set_error("cudaStreamCreate failed: %s", cudaGetErrorString(e));
            delete j;
            return GPUNMF_ERR_CUDA;
        }
        j->own_stream = true;
    }
    if (!j->async_alloc) {  // a public job: the library's pool (where the device has one)
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess) j->pool = library_pool(dev);
    }
    Sizes z = compute_sizes(rule, n, m, r, precision);
    j->s_h = z.s_h; j->s_w = z.s_w; j->s_g = z.s_g;
    gpunmf_status st = GPUNMF_OK;
#define ALLOC(ptr, cnt) \
    if (st == GPUNMF_OK) st = dalloc(j, &(ptr), (cnt));
    ALLOC(j->V, (size_t)n * m);
    ALLOC(j->W, (size_t)n * r);
    ALLOC(j->H, (size_t)r * m);
    ALLOC(j->P_h, z.p_h);
    ALLOC(j->P_w, z.p_w);
    ALLOC(j->P_g, z.p_g);
    ALLOC(j->G, (size_t)r * r);
    ALLOC(j->D_h, z.d_h);
    ALLOC(j->D_w, z.d_w);
    ALLOC(j->WH, z.wh);
    ALLOC(j->sums, (size_t)r);
    ALLOC(j->d_quality, 4);
    ALLOC(j->red, z.red);
    ALLOC(j->d_scalar, 4);
#undef ALLOC
    j->red_cap = z.red;
    if (st == GPUNMF_OK && pinned64) {
        j->h_pinned = pinned64;
        j->external_pinned = true;
        memset(j->h_pinned, 0, 64);
    } else if (st == GPUNMF_OK) {
        cudaError_t e = cudaHostAlloc((void **)&j->h_pinned, 64, cudaHostAllocDefault);
        if (e != cudaSuccess) {
            set_error("cudaHostAlloc failed: %s", cudaGetErrorString(e));
            st = GPUNMF_ERR_NOMEM;
        } else {
            memset(j->h_pinned, 0, 64);
        }
    }
    if (st == GPUNMF_OK) {
        cudaError_t e = cudaEventCreateWithFlags(&j->qev, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            set_error("cudaEventCreate failed: %s", cudaGetErrorString(e));
            st = GPUNMF_ERR_CUDA;
        }
    }
    if (st == GPUNMF_OK && precision == GPUNMF_BF16) st = tc_create(j);
    if (st != GPUNMF_OK) {
        job_free(j);
        return st;
    }
    // quality bookkeeping as constructed in nmf_base.h:94-97,116-119
    j->q_interval = 1;
    j->q_times = 0;
    j->q_delta = 1.0f;
    j->q_last = -1.0f;
    j->h_quality()[0] = 0.0f;
    *out = j;
    return GPUNMF_OK;
}

// The address at which kernels of the current device read host matrix p, or null: page-locked
// memory mapped into the device's address space.  (Pageable memory is readable too where the device
// uses the host page tables, but the conversion kernel's reads of it ran at ~116 GB/s against
// ~210 GB/s for a copy, so pageable matrices are copied first.)
static const float *device_readable_host(const float *p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) == cudaSuccess && a.type == cudaMemoryTypeHost && a.devicePointer)
        return static_cast<const float *>(a.devicePointer);
    cudaGetLastError();
    return nullptr;
}

static gpunmf_status job_upload(gpunmf_job *j, const float *V, const float *W, const float *H, cudaMemcpyKind kind) {
    size_t nm = (size_t)j->n * j->m, nr = (size_t)j->n * j->r, rm = (size_t)j->r * j->m;
    // BF16 jobs from page-locked host memory: V crosses the host link once, read by the conversion
    // kernel that writes its BF16 copies and the FP32 copy (a copy first and a conversion after
    // would move V through device memory twice more)
    const float *v_src = (kind == cudaMemcpyHostToDevice && j->precision == GPUNMF_BF16) ? device_readable_host(V)
                                                                                        : nullptr;
    if (!v_src) GPUNMF_CUDA_TRY(cudaMemcpyAsync(j->V, V, nm * sizeof(float), kind, j->stream));
    GPUNMF_CUDA_TRY(cudaMemcpyAsync(j->W, W, nr * sizeof(float), kind, j->stream));
    GPUNMF_CUDA_TRY(cudaMemcpyAsync(j->H, H, rm * sizeof(float), kind, j->stream));
    if (j->precision == GPUNMF_BF16) TRY_STATUS(tc_prepare(j, v_src));
    return GPUNMF_OK;
}

// ------------------------------------------------------------------------
// quality bookkeeping (nmf_base.h:70-89).  By default made deterministic:
// instead of sampling only when the previous asynchronous read-back happens to
// be complete, every k-th iteration samples and the previous read-back is
// waited for.  Interval GPUNMF_QUALITY_WHEN_READY keeps the reference's own
// rule: an iteration samples only if the previous read-back is complete
// (nmf_base.h:71, cudaStreamQuery on the read-back's stream), and never waits.
// ------------------------------------------------------------------------
static gpunmf_status quality_step(gpunmf_job *j, bool fused_wh) {
    if (j->q_interval == 0) return GPUNMF_OK;
    if (j->q_interval > 0 && (j->iter_count % j->q_interval) != 0) return GPUNMF_OK;
    if (j->q_pending) {
        if (j->q_interval == GPUNMF_QUALITY_WHEN_READY) {
            const cudaError_t e = cudaEventQuery(j->qev);
            if (e == cudaErrorNotReady) {
                if (cudaPeekAtLastError() == cudaErrorNotReady) cudaGetLastError();  // not an error
                return GPUNMF_OK;
            }
            GPUNMF_CUDA_TRY(e);
        } else {
            GPUNMF_CUDA_TRY(cudaEventSynchronize(j->qev));
        }
        j->q_pending = false;
    }
    float quality = j->h_quality()[0];
    if (j->q_times++ > 2) {
        j->q_delta = quality - j->q_last;
    } else {
        j->q_times++;
    }
    j->q_last = quality;
    cudaStream_t s = j->stream;
    int n = j->n, m = j->m, r = j->r;
    // BF16 jobs whose H-step can carry the sample: no launch of its own (the H-step records the event)
    if (j->precision == GPUNMF_BF16 && tc_quality_fold(j)) return GPUNMF_OK;
    if (j->precision == GPUNMF_BF16 && tc_quality_ready(j)) {
        // BF16 jobs: W H on the tensor cores from the BF16 factors, V as BF16; one launch that also
        // writes the value into the pinned read-back word where the device can reach it
        TRY_STATUS(tc_quality(j));
        if (!tc_quality_writes_host(j))
            GPUNMF_CUDA_TRY(cudaMemcpyAsync(j->h_quality(), j->d_quality, sizeof(float), cudaMemcpyDeviceToHost, s));
        GPUNMF_CUDA_TRY(cudaEventRecord(j->qev, s));
        j->q_pending = true;
        return GPUNMF_OK;
    } else if (fused_wh) {
        GPUNMF_CUDA_TRY(wh_quality_f32(n, m, r, j->W, j->H, j->V, j->eps, j->red, s));
        GPUNMF_CUDA_TRY(finalize_partials(j->red, wh_reduce_ctas(n, m), 1, 0, j->d_quality, nullptr, s));
    } else {
        long long cnt = (long long)n * m;
        GPUNMF_CUDA_TRY(quality_ew(j->V, j->WH, cnt, j->eps, j->red, s));
        GPUNMF_CUDA_TRY(finalize_partials(j->red, quality_ew_ctas(cnt), 1, 0, j->d_quality, nullptr, s));
    }
    j->launches += 2;
    GPUNMF_CUDA_TRY(cudaMemcpyAsync(j->h_quality(), j->d_quality, sizeof(float), cudaMemcpyDeviceToHost, s));
    GPUNMF_CUDA_TRY(cudaEventRecord(j->qev, s));
    j->q_pending = true;
    return GPUNMF_OK;
}

// kernel-timing hooks around the V-streaming products
void mark_begin(gpunmf_job *j) {
    if (!j->timing) return;
    cudaEvent_t e;
    if (cudaEventCreate(&e) == cudaSuccess) {
        cudaEventRecord(e, j->stream);
        j->tev.push_back(e);
    }
}
void mark_end(gpunmf_job *j) {
    if (!j->timing) return;
    cudaEvent_t e;
    if (cudaEventCreate(&e) == cudaSuccess) {
        cudaEventRecord(e, j->stream);
        j->tev.push_back(e);
    }
    j->timed_launches++;
}

// ------------------------------------------------------------------------
// FP32 iterations
// ------------------------------------------------------------------------
static gpunmf_status iterate_euclid_f32(gpunmf_job *j, bool updateW) {
    const int n = j->n, m = j->m, r = j->r;
    cudaStream_t s = j->stream;
    const bool additive = j->rule != GPUNMF_EUCLIDEAN;
    TRY_STATUS(quality_step(j, true));
    if (j->rule != GPUNMF_ADDITIVE_EUCLIDEAN_FIXED_H) {
        // H <- H .* (W'V) ./ (W'W H + eps)   or the additive step on the same products
        mark_begin(j);
        GPUNMF_CUDA_TRY(gemm_f32(r, m, n, {j->W, n, true}, {j->V, n, false}, j->P_h, r, j->s_h, s));
        mark_end(j);
        int sg = gemm_f32_splits(r, r, n);
        GPUNMF_CUDA_TRY(gemm_f32(r, r, n, {j->W, n, true}, {j->W, n, false}, sg > 1 ? j->P_g : j->G, r, sg, s));
        if (sg > 1) GPUNMF_CUDA_TRY(sum_partials(j->G, j->P_g, sg, (long long)r * r, s));
        GPUNMF_CUDA_TRY(gemm_f32(r, m, r, {j->G, r, false}, {j->H, r, false}, j->D_h, r, 1, s));
        if (additive)
            GPUNMF_CUDA_TRY(additive_update(j->H, j->P_h, j->s_h, j->D_h, (long long)r * m, s));
        else
            GPUNMF_CUDA_TRY(euclid_update(j->H, j->P_h, j->s_h, j->D_h, (long long)r * m, j->eps, s));
        j->launches += 4 + (sg > 1);
    }
    if (!updateW) return GPUNMF_OK;
    // W <- W .* (V H') ./ (W H H' + eps)   or the additive step on the same products
    mark_begin(j);
    GPUNMF_CUDA_TRY(gemm_f32(n, r, m, {j->V, n, false}, {j->H, r, true}, j->P_w, n, j->s_w, s));
    mark_end(j);
    const int sgw = gemm_f32_splits(r, r, m);
    GPUNMF_CUDA_TRY(gemm_f32(r, r, m, {j->H, r, false}, {j->H, r, true}, sgw > 1 ? j->P_g : j->G, r, sgw, s));
    if (sgw > 1) GPUNMF_CUDA_TRY(sum_partials(j->G, j->P_g, sgw, (long long)r * r, s));
    GPUNMF_CUDA_TRY(gemm_f32(n, r, r, {j->W, n, false}, {j->G, r, false}, j->D_w, n, 1, s));
    if (additive)
        GPUNMF_CUDA_TRY(additive_update(j->W, j->P_w, j->s_w, j->D_w, (long long)n * r, s));
    else
        GPUNMF_CUDA_TRY(euclid_update(j->W, j->P_w, j->s_w, j->D_w, (long long)n * r, j->eps, s));
    j->launches += 4 + (sgw > 1);
    return GPUNMF_OK;
}

static gpunmf_status iterate_kl_f32(gpunmf_job *j, bool updateW) {
    const int n = j->n, m = j->m, r = j->r;
    cudaStream_t s = j->stream;
    const bool additive = j->rule == GPUNMF_ADDITIVE_DIVERGENCE;
    GPUNMF_CUDA_TRY(gemm_f32(n, m, r, {j->W, n, false}, {j->H, r, false}, j->WH, n, 1, s));
    j->launches++;
    TRY_STATUS(quality_step(j, false));
    GPUNMF_CUDA_TRY(col_sums(j->W, n, r, j->eps, j->sums, s));
    mark_begin(j);
    GPUNMF_CUDA_TRY(
        gemm_f32_ratio_right(r, m, n, {j->W, n, true}, j->V, j->WH, n, j->eps, j->P_h, j->s_h, s, additive));
    mark_end(j);
    GPUNMF_CUDA_TRY(kl_update(j->H, j->P_h, j->s_h, j->sums, (long long)r * m, 1, r, s, additive));
    j->launches += 3;
    if (!updateW) return GPUNMF_OK;
    GPUNMF_CUDA_TRY(gemm_f32(n, m, r, {j->W, n, false}, {j->H, r, false}, j->WH, n, 1, s));
    GPUNMF_CUDA_TRY(row_sums(j->H, r, m, j->eps, j->sums, s));
    mark_begin(j);
    GPUNMF_CUDA_TRY(
        gemm_f32_ratio_left(n, r, m, j->V, j->WH, n, j->eps, {j->H, r, true}, j->P_w, j->s_w, s, additive));
    mark_end(j);
    GPUNMF_CUDA_TRY(kl_update(j->W, j->P_w, j->s_w, j->sums, (long long)n * r, n, r, s, additive));
    j->launches += 4;
    return GPUNMF_OK;
}

static gpunmf_status job_iterate(gpunmf_job *j, int iters, bool updateW) {
    for (int it = 0; it < iters; it++) {
        gpunmf_status st;
        if (j->precision == GPUNMF_BF16)
            st = tc_iterate(j, updateW);
        else if (rule_is_kl(j->rule))
            st = iterate_kl_f32(j, updateW);
        else
            st = iterate_euclid_f32(j, updateW);
        if (st != GPUNMF_OK) return st;
        j->iter_count++;
    }
    return GPUNMF_OK;
}

gpunmf_status job_quality_step(gpunmf_job *j, bool fused_wh) { return quality_step(j, fused_wh); }

static gpunmf_status ensure_wh(gpunmf_job *j) {
    if (!j->WH) TRY_STATUS(dalloc(j, &j->WH, (size_t)j->n * j->m));
    GPUNMF_CUDA_TRY(gemm_f32(j->n, j->m, j->r, {j->W, j->n, false}, {j->H, j->r, false}, j->WH, j->n, 1, j->stream));
    return GPUNMF_OK;
}

gpunmf_status job_create_empty(int rule, int n, int m, int r, float eps, int precision, cudaStream_t stream,
                               unsigned char *pinned64, bool async_alloc, gpunmf_job **out, int cta_cap) {
    return job_alloc(rule, n, m, r, eps, precision, (void *)stream, out, pinned64, async_alloc, cta_cap);
}

gpunmf_status job_prepare(gpunmf_job *j) {
    if (j->precision == GPUNMF_BF16) return tc_prepare(j);
    return GPUNMF_OK;
}

gpunmf_status job_run(gpunmf_job *j, int iters, bool updateW) { return job_iterate(j, iters, updateW); }

void job_release(gpunmf_job *j) { job_free(j); }

}  // namespace gpunmf

using namespace gpunmf;

// ------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------
#define CHECK_HANDLE(h)                     \
    do {                                    \
        if (!(h)) {                         \
            set_error("null handle");       \
            return GPUNMF_ERR_INVALID;      \
        }                                   \
    } while (0)

extern "C" {

const char *gpunmf_last_error(void) { return g_err; }

const char *gpunmf_version(void) { return "gpunmf 0.1 (sm_103a)"; }

int gpunmf_device_count(void) {
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return c;
}

gpunmf_status gpunmf_create(int rule, int n, int m, int r, const float *V, const float *W, const float *H,
                            float eps, int precision, void *stream, gpunmf_handle *out) {
    if (!out || !V || !W || !H) {
        set_error("null argument");
        return GPUNMF_ERR_INVALID;
    }
    gpunmf_job *j;
    TRY_STATUS(job_alloc(rule, n, m, r, eps, precision, stream, &j));
    gpunmf_status st = job_upload(j, V, W, H, cudaMemcpyHostToDevice);
    if (st == GPUNMF_OK) {
        cudaError_t e = cudaStreamSynchronize(j->stream);  // host buffers may be released on return
        if (e != cudaSuccess) {
            set_error("upload failed: %s", cudaGetErrorString(e));
            st = GPUNMF_ERR_CUDA;
        }
    }
    if (st != GPUNMF_OK) {
        job_free(j);
        return st;
    }
    *out = j;
    return GPUNMF_OK;
}

gpunmf_status gpunmf_create_device(int rule, int n, int m, int r, const float *dV, const float *dW,
                                   const float *dH, float eps, int precision, void *stream,
                                   gpunmf_handle *out) {
    if (!out || !dV || !dW || !dH) {
        set_error("null argument");
        return GPUNMF_ERR_INVALID;
    }
    gpunmf_job *j;
    TRY_STATUS(job_alloc(rule, n, m, r, eps, precision, stream, &j));
    gpunmf_status st = job_upload(j, dV, dW, dH, cudaMemcpyDeviceToDevice);
    if (st != GPUNMF_OK) {
        job_free(j);
        return st;
    }
    *out = j;
    return GPUNMF_OK;
}

static inline float uniform_from_counter(unsigned long long key, unsigned long long idx) {
    // splitmix64 finaliser over (key + (idx+1) * golden gamma); top 24 bits -> [0,1)
    unsigned long long z = key + (idx + 1ULL) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (float)(z >> 40) * (1.0f / 16777216.0f);
}

void gpunmf_fill_uniform(unsigned long long seed, unsigned long long offset, size_t count, float *out) {
    if (!out) return;
    unsigned long long key = seed * 0xD1B54A32D192ED03ULL + 0x8CB92BA72F3D8DD7ULL;
    for (size_t k = 0; k < count; k++) out[k] = uniform_from_counter(key, offset + k);
}

void *gpunmf_host_alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        set_error("cudaHostAlloc of %zu bytes failed", bytes);
        return nullptr;
    }
    return p;
}

void gpunmf_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

gpunmf_status gpunmf_create_random(int rule, int n, int m, int r, const float *V, unsigned long long seed,
                                   float eps, int precision, void *stream, gpunmf_handle *out) {
    if (!out || !V || n <= 0 || m <= 0 || r <= 0) {
        set_error("invalid argument");
        return GPUNMF_ERR_INVALID;
    }
    // NMF::Randomize (nmf_base.h:56-61): uniform[0,1) + eps, W first then H
    std::vector<float> W((size_t)n * r), H((size_t)r * m);
    gpunmf_fill_uniform(seed, 0, W.size(), W.data());
    gpunmf_fill_uniform(seed, W.size(), H.size(), H.data());
    for (float &x : W) x += eps;
    for (float &x : H) x += eps;
    return gpunmf_create(rule, n, m, r, V, W.data(), H.data(), eps, precision, stream, out);
}

gpunmf_status gpunmf_trim_pool(void) {
    int dev = 0;
    GPUNMF_CUDA_TRY(cudaGetDevice(&dev));
    cudaMemPool_t pool = library_pool(dev);
    if (pool) GPUNMF_CUDA_TRY(cudaMemPoolTrimTo(pool, 0));
    return GPUNMF_OK;
}

gpunmf_status gpunmf_destroy(gpunmf_handle h) {
    CHECK_HANDLE(h);
    if (h->stream) cudaStreamSynchronize(h->stream);
    job_free(h);
    return GPUNMF_OK;
}

gpunmf_status gpunmf_iterate(gpunmf_handle h, int iters, int updateW) {
    CHECK_HANDLE(h);
    if (iters < 0) {
        set_error("iters must be >= 0");
        return GPUNMF_ERR_INVALID;
    }
    return job_iterate(h, iters, updateW != 0);
}

gpunmf_status gpunmf_set_quality_interval(gpunmf_handle h, int interval) {
    CHECK_HANDLE(h);
    if (interval < 0 && interval != GPUNMF_QUALITY_WHEN_READY) {
        set_error("interval must be >= 0 or GPUNMF_QUALITY_WHEN_READY (-1)");
        return GPUNMF_ERR_INVALID;
    }
    h->q_interval = interval;
    return GPUNMF_OK;
}

gpunmf_status gpunmf_set_wait_limit_cycles(gpunmf_handle h, long long cycles) {
    CHECK_HANDLE(h);
    if (h->precision != GPUNMF_BF16) {
        set_error("only the BF16 tensor-core kernels wait on one another");
        return GPUNMF_ERR_UNSUPPORTED;
    }
    tc_set_wait_limit(h, cycles);
    return GPUNMF_OK;
}

gpunmf_status gpunmf_inject_missing_arrival(gpunmf_handle h) {
    CHECK_HANDLE(h);
    if (h->precision != GPUNMF_BF16) {
        set_error("only the BF16 tensor-core kernels count tile arrivals");
        return GPUNMF_ERR_UNSUPPORTED;
    }
    return tc_inject_missing_arrival(h);
}

gpunmf_status gpunmf_set_grid_limit(int ctas) {
    if (ctas < 0) {
        set_error("grid limit must be >= 0");
        return GPUNMF_ERR_INVALID;
    }
    tc_set_grid_limit(ctas);
    return GPUNMF_OK;
}

gpunmf_status gpunmf_quality_improvement(gpunmf_handle h, float *out) {
    CHECK_HANDLE(h);
    if (!out) return GPUNMF_ERR_INVALID;
    *out = h->q_delta;
    return GPUNMF_OK;
}

gpunmf_status gpunmf_residual_fp64(gpunmf_handle h, double *out) {
    CHECK_HANDLE(h);
    if (!out) return GPUNMF_ERR_INVALID;
    cudaStream_t s = h->stream;
    GPUNMF_CUDA_TRY(wh_residual_f32(h->n, h->m, h->r, h->W, h->H, h->V, h->red, s));
    GPUNMF_CUDA_TRY(finalize_partials(h->red, wh_reduce_ctas(h->n, h->m), 2, 1, nullptr, h->d_scalar, s));
    GPUNMF_CUDA_TRY(cudaMemcpyAsync(h->h_scalar(), h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, s));
    GPUNMF_CUDA_TRY(cudaStreamSynchronize(s));
    *out = h->h_scalar()[0];
    return tc_check(h);
}

gpunmf_status gpunmf_objective_kl_fp64(gpunmf_handle h, double *out) {
    CHECK_HANDLE(h);
    if (!out) return GPUNMF_ERR_INVALID;
    cudaStream_t s = h->stream;
    TRY_STATUS(ensure_wh(h));
    long long cnt = (long long)h->n * h->m;
    int ctas = quality_ew_ctas(cnt);
    if ((size_t)ctas > h->red_cap) {
        set_error("reduction buffer too small");
        return GPUNMF_ERR_INVALID;
    }
    GPUNMF_CUDA_TRY(kl_objective_ew(h->V, h->WH, cnt, h->red, s));
    GPUNMF_CUDA_TRY(finalize_partials(h->red, ctas, 1, 0, nullptr, h->d_scalar, s));
    GPUNMF_CUDA_TRY(cudaMemcpyAsync(h->h_scalar(), h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, s));
    GPUNMF_CUDA_TRY(cudaStreamSynchronize(s));
    *out = h->h_scalar()[0];
    return GPUNMF_OK;
}

gpunmf_status gpunmf_get_w(gpunmf_handle h, float *W) {
    CHECK_HANDLE(h);
    if (!W) return GPUNMF_ERR_INVALID;
    GPUNMF_CUDA_TRY(cudaMemcpyAsync(W, h->W, sizeof(float) * (size_t)h->n * h->r, cudaMemcpyDeviceToHost, h->stream));
    GPUNMF_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return tc_check(h);
}

gpunmf_status gpunmf_get_h(gpunmf_handle h, float *H) {
    CHECK_HANDLE(h);
    if (!H) return GPUNMF_ERR_INVALID;
    GPUNMF_CUDA_TRY(cudaMemcpyAsync(H, h->H, sizeof(float) * (size_t)h->r * h->m, cudaMemcpyDeviceToHost, h->stream));
    GPUNMF_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return tc_check(h);
}

gpunmf_status gpunmf_get_wh(gpunmf_handle h, float *WH) {
    CHECK_HANDLE(h);
    if (!WH) return GPUNMF_ERR_INVALID;
    TRY_STATUS(ensure_wh(h));
    GPUNMF_CUDA_TRY(cudaMemcpyAsync(WH, h->WH, sizeof(float) * (size_t)h->n * h->m, cudaMemcpyDeviceToHost, h->stream));
    GPUNMF_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return GPUNMF_OK;
}

gpunmf_status gpunmf_device_factors(gpunmf_handle h, float **dW, float **dH) {
    CHECK_HANDLE(h);
    if (dW) *dW = h->W;
    if (dH) *dH = h->H;
    return GPUNMF_OK;
}

gpunmf_status gpunmf_synchronize(gpunmf_handle h) {
    CHECK_HANDLE(h);
    GPUNMF_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return tc_check(h);
}

gpunmf_status gpunmf_info(gpunmf_handle h, int *rule, int *n, int *m, int *r, int *precision, float *eps) {
    CHECK_HANDLE(h);
    if (rule) *rule = h->rule;
    if (n) *n = h->n;
    if (m) *m = h->m;
    if (r) *r = h->r;
    if (precision) *precision = h->precision;
    if (eps) *eps = h->eps;
    return GPUNMF_OK;
}

size_t gpunmf_footprint_bytes(int rule, int n, int m, int r, int precision) {
    if (n <= 0 || m <= 0 || r <= 0) return 0;
    return job_footprint(rule, n, m, r, precision);
}

gpunmf_status gpunmf_time_iterations(gpunmf_handle h, int iters, int updateW, float *total_ms, float *kernel_ms,
                                     int *kernel_launches, int *all_launches) {
    CHECK_HANDLE(h);
    if (iters < 0) return GPUNMF_ERR_INVALID;
    cudaEvent_t e0, e1;
    GPUNMF_CUDA_TRY(cudaEventCreate(&e0));
    GPUNMF_CUDA_TRY(cudaEventCreate(&e1));
    for (cudaEvent_t e : h->tev) cudaEventDestroy(e);
    h->tev.clear();
    h->timed_launches = 0;
    h->timing = kernel_ms != nullptr;
    long long l0 = h->launches;
    gpunmf_status st = GPUNMF_OK;
    cudaError_t ce = cudaEventRecord(e0, h->stream);
    if (ce == cudaSuccess) st = job_iterate(h, iters, updateW != 0);
    if (ce == cudaSuccess) ce = cudaEventRecord(e1, h->stream);
    if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
    h->timing = false;
    float ms = 0.f;
    if (ce == cudaSuccess && st == GPUNMF_OK) ce = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ce != cudaSuccess) {
        set_error("timing failed: %s", cudaGetErrorString(ce));
        return GPUNMF_ERR_CUDA;
    }
    if (st != GPUNMF_OK) return st;
    st = tc_check(h);
    if (st != GPUNMF_OK) return st;
    if (total_ms) *total_ms = ms;
    if (kernel_ms) {
        float acc = 0.f;
        for (size_t k = 0; k + 1 < h->tev.size(); k += 2) {
            float t = 0.f;
            if (cudaEventElapsedTime(&t, h->tev[k], h->tev[k + 1]) == cudaSuccess) acc += t;
        }
        *kernel_ms = acc;
    }
    if (kernel_launches) *kernel_launches = h->timed_launches;
    if (all_launches) *all_launches = (int)(h->launches - l0);
    for (cudaEvent_t e : h->tev) cudaEventDestroy(e);
    h->tev.clear();
    return GPUNMF_OK;
}

}  // extern "C"
