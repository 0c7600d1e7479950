// Internal job structure shared by the engine and the tensor-core path.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "../../include/gpunmf.h"

struct TcState;  // tensor-core path state (tc_kernels.cu)

struct gpunmf_job {
    int rule = 0, n = 0, m = 0, r = 0, precision = 0;
    float eps = 1e-8f;
    int cta_cap = 0;  // CTAs per launch of the tensor-core kernels at most (0: the SMs)
    cudaStream_t stream = nullptr;
    bool own_stream = false;

    // FP32 master copies, column-major (V n x m, W n x r, H r x m)
    float *V = nullptr, *W = nullptr, *H = nullptr;

    // FP32-path workspaces
    int s_h = 1, s_w = 1, s_g = 1;            // split-K slices
    float *P_h = nullptr, *P_w = nullptr;     // split-K partial products of the H- and W-steps
    float *P_g = nullptr, *G = nullptr;       // Gram partials, Gram (r x r)
    float *D_h = nullptr, *D_w = nullptr;     // W'W H (r x m) and W H H' (n x r)
    float *WH = nullptr;                      // n x m (KL; lazily for GetWH)
    float *sums = nullptr;                    // r (KL column/row sums)
    double *red = nullptr;                    // per-CTA FP64 partials
    size_t red_cap = 0;
    float *d_quality = nullptr;
    double *d_scalar = nullptr;
    unsigned char *h_pinned = nullptr;        // 64 pinned bytes: quality (float) at 0, scalar (double) at 8
    float *h_quality() { return reinterpret_cast<float *>(h_pinned); }
    double *h_scalar() { return reinterpret_cast<double *>(h_pinned + 8); }

    // quality bookkeeping (src/algorithms/nmf/nmf_base.h:49-53)
    int q_interval = 1;
    int q_times = 0;
    float q_last = -1.0f, q_delta = 1.0f;
    bool q_pending = false;
    cudaEvent_t qev = nullptr;
    long long iter_count = 0;

    // launch accounting and optional per-kernel timing
    long long launches = 0;
    bool timing = false;
    int timed_launches = 0;
    std::vector<cudaEvent_t> tev;

    TcState *tc = nullptr;

    // allocation mode: jobs made by the server use the stream-ordered allocator on their
    // stream (no device-wide synchronisation on free) and a pinned block owned by the server
    bool async_alloc = false;
    // public jobs: device memory stream-ordered from the library's pool, which keeps freed blocks
    // for the next job (creating a job then makes no driver allocation once the pool has grown)
    cudaMemPool_t pool = nullptr;
    bool external_pinned = false;
};

namespace gpunmf {
// rule families: the Euclidean rules share products (W'V, W'W H, V H', W H H'), the KL rules a
// stored WH and the ratio V/(WH+eps)
inline bool rule_valid(int rule) { return rule >= GPUNMF_EUCLIDEAN && rule <= GPUNMF_ADDITIVE_EUCLIDEAN_FIXED_H; }
inline bool rule_is_kl(int rule) { return rule == GPUNMF_DIVERGENCE || rule == GPUNMF_ADDITIVE_DIVERGENCE; }
inline bool rule_is_additive(int rule) { return rule >= GPUNMF_ADDITIVE_EUCLIDEAN; }
// device memory of a job: cudaMalloc / cudaFree, or cudaMallocAsync / cudaFreeAsync on the job's stream
cudaError_t job_dev_alloc(gpunmf_job *j, void **p, size_t bytes);
void job_dev_free(gpunmf_job *j, void *p);
// host -> device copy of set-up data (synchronous, or ordered on the job's stream)
cudaError_t job_h2d(gpunmf_job *j, void *dst, const void *src, size_t bytes);
// a job without data (the caller fills V, W, H on the job's stream, then calls job_prepare)
gpunmf_status job_create_empty(int rule, int n, int m, int r, float eps, int precision, cudaStream_t stream,
                               unsigned char *pinned64, bool async_alloc, gpunmf_job **out, int cta_cap = 0);
gpunmf_status job_prepare(gpunmf_job *j);
gpunmf_status job_run(gpunmf_job *j, int iters, bool updateW);
void job_release(gpunmf_job *j);  // frees without synchronising (stream-ordered when async_alloc)
void mark_begin(gpunmf_job *j);
void mark_end(gpunmf_job *j);
gpunmf_status job_quality_step(gpunmf_job *j, bool fused_wh);
size_t job_footprint(int rule, int n, int m, int r, int precision);

// tensor-core path (tc_kernels.cu)
gpunmf_status tc_supported(int rule, int n, int m, int r);
void tc_add_sizes(int rule, int n, int m, int r, size_t *red_doubles);
size_t tc_footprint(int rule, int n, int m, int r);
gpunmf_status tc_create(gpunmf_job *j);
// after V/W/H are uploaded; or, with v_src (V in host memory the device can read), after W/H are:
// then the BF16 conversion reads V from there and also writes the job's FP32 V
gpunmf_status tc_prepare(gpunmf_job *j, const float *v_src = nullptr);
gpunmf_status tc_iterate(gpunmf_job *j, bool updateW);
// quality of the current factors on the tensor cores (BF16 jobs with npad <= 128)
bool tc_quality_ready(const gpunmf_job *j);
// whether the tensor-core quality kernel writes the job's pinned read-back word itself
bool tc_quality_writes_host(const gpunmf_job *j);
gpunmf_status tc_quality(gpunmf_job *j);
// fused Euclidean jobs: the next H-step launch samples the quality itself (it also records the
// job's quality event); false where it cannot
bool tc_quality_fold(gpunmf_job *j);
gpunmf_status tc_check(gpunmf_job *j);    // reads the kernels' error word (after a sync)
void tc_set_wait_limit(gpunmf_job *j, long long cycles);  // <= 0: the default (about 2 s)
gpunmf_status tc_inject_missing_arrival(gpunmf_job *j);
void tc_set_grid_limit(int ctas);         // CTAs per launch of jobs created later (0: one per SM)
void tc_destroy(gpunmf_job *j);
}  // namespace gpunmf
