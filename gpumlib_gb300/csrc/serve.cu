// NMF serving with continuous batching.
//
// Jobs (rule, n, m, r, seed) arrive at any time.  A scheduler thread admits a
// pending job as soon as a stream slot is free and its device footprint fits
// the HBM budget, then advances every admitted job in chunks of iterations,
// each chunk followed by an FP64 relative-residual check whose result comes
// back asynchronously (pinned read-back + event).  A job retires at residual
// <= tol or after max_iters iterations; its slot and memory go to the next
// pending job at once.  Jobs run on their own streams, so the kernels of all
// admitted jobs overlap on the device, and each job's arithmetic is the same
// as when it runs alone (same kernels, same order on its own stream).
//
// Job data is generated on the device from the job's seed
// (V = A B + |N(0, sigma)|, A n x r and B r x m uniform[0,1); W, H
// uniform[0,1) + 1e-4), standing in for matrices that arrive in device memory
// from an upstream stage.  Device memory comes from the stream-ordered
// allocator so that retiring a job never synchronises the device.
#include <math.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "engine.h"
#include "kernels.h"

namespace gpunmf {

// counter-based uniform in [0,1) (splitmix64 finaliser), same key schedule as the host generator
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
__device__ __forceinline__ float dev_uniform(unsigned long long key, unsigned long long idx) {
    return (float)(mix64(key + (idx + 1ULL) * 0x9E3779B97F4A7C15ULL) >> 40) * (1.0f / 16777216.0f);
}
__host__ __device__ __forceinline__ unsigned long long stream_key(unsigned long long seed, unsigned stream) {
    return (seed * 0xD1B54A32D192ED03ULL + 0x8CB92BA72F3D8DD7ULL) ^ ((unsigned long long)stream << 56);
}

__global__ void gen_uniform_kernel(float *x, long long count, unsigned long long key, float add) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
         k += (long long)gridDim.x * blockDim.x)
        x[k] = dev_uniform(key, k) + add;
}

// V += |sigma * N(0,1)|, Box-Muller on two counter uniforms
__global__ void add_abs_noise_kernel(float *V, long long count, unsigned long long key, float sigma) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
         k += (long long)gridDim.x * blockDim.x) {
        float u1 = dev_uniform(key, 2 * k) + (0.5f / 16777216.0f);
        float u2 = dev_uniform(key, 2 * k + 1);
        float z = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
        V[k] += fabsf(sigma * z);
    }
}

static int gen_blocks(long long count) {
    long long b = (count + 255) / 256;
    return (int)std::min<long long>(std::max<long long>(b, 1), 4 * kNumSMsGB300);
}

// V (n x m), W (n x r), H (r x m) of a job with this seed, on stream s (W and H hold A and B while
// V = A B is formed)
static gpunmf_status generate_data(int n, int m, int r, unsigned long long seed, float sigma, float *V, float *W,
                                   float *H, cudaStream_t s) {
    const long long nr = (long long)n * r, rm = (long long)r * m, nm = (long long)n * m;
    gen_uniform_kernel<<<gen_blocks(nr), 256, 0, s>>>(W, nr, stream_key(seed, 0), 0.f);   // A
    gen_uniform_kernel<<<gen_blocks(rm), 256, 0, s>>>(H, rm, stream_key(seed, 1), 0.f);   // B
    GPUNMF_CUDA_TRY(cudaGetLastError());
    GPUNMF_CUDA_TRY(gemm_f32(n, m, r, {W, n, false}, {H, r, false}, V, n, 1, s));
    add_abs_noise_kernel<<<gen_blocks(nm), 256, 0, s>>>(V, nm, stream_key(seed, 2), sigma);
    gen_uniform_kernel<<<gen_blocks(nr), 256, 0, s>>>(W, nr, stream_key(seed, 3), 1e-4f);
    gen_uniform_kernel<<<gen_blocks(rm), 256, 0, s>>>(H, rm, stream_key(seed, 4), 1e-4f);
    GPUNMF_CUDA_TRY(cudaGetLastError());
    return GPUNMF_OK;
}

// fills j->V, j->W, j->H on the job's stream
static gpunmf_status generate_job_data(gpunmf_job *j, unsigned long long seed, float sigma) {
    return generate_data(j->n, j->m, j->r, seed, sigma, j->V, j->W, j->H, j->stream);
}

}  // namespace gpunmf

using namespace gpunmf;

struct SJob {
    gpunmf_server_result res{};
    unsigned long long seed = 0;
    float eps = 1e-8f;
    size_t footprint = 0;
    gpunmf_job *job = nullptr;
    int slot = -1;
    bool check_pending = false;
    cudaGraphExec_t chunk_graph = nullptr;  // one full chunk + residual check, captured at admission
    std::vector<float> W, H;  // kept factors (keep_factors mode)
};

// CTAs per launch of a served BF16 job's tensor-core kernels: its 128 x 128 blocks per half-step
// divided by kServeBlocksPerCta, at least one and at most kServeMaxJobCtas.  A job created alone
// takes one CTA per block up to every SM; in the server the large jobs' grids are capped so that
// they leave SMs to the jobs running beside them.  Measured on the 2000 jobs/s stream (1 s of it,
// 1970 jobs, 64 slots): every SM 155 jobs/s, at most 48 CTAs 249, 24 CTAs 306, 12 CTAs 118 (the
// large jobs then take too long); more than one block per CTA costs more per job than the
// concurrency gains (8 blocks per CTA: 23 jobs/s), since the kernels are built for about one
// block per CTA.
constexpr int kServeBlocksPerCta = 1;
constexpr int kServeMaxJobCtas = 24;

struct gpunmf_server {
    int device = 0;
    std::atomic<int> blocks_per_cta{kServeBlocksPerCta}, max_job_ctas{kServeMaxJobCtas};
    int slots = 0, precision = 0, check_every = 10, max_iters = 500;
    size_t budget = 0, in_use = 0;
    double tol = 1e-3;
    float sigma = 0.01f;
    bool keep = false;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;
    double *d_res = nullptr, *h_res = nullptr;
    unsigned char *h_pin = nullptr;
    std::vector<int> free_slots;
    std::vector<SJob *> slot_job;
    std::deque<SJob *> pending;
    std::vector<SJob *> done;
    long long submitted = 0, finished = 0;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv, cv_done;
    bool stop = false;
    std::string fatal;
    std::chrono::steady_clock::time_point t0;
    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

// the work of one chunk on the job's stream: `chunk` iterations, then the residual into h_res[slot]
static gpunmf_status chunk_body(gpunmf_server *S, SJob *q, int chunk) {
    gpunmf_job *j = q->job;
    gpunmf_status st = job_run(j, chunk, true);
    if (st != GPUNMF_OK) return st;
    cudaStream_t s = j->stream;
    const int ctas = wh_reduce_ctas(j->n, j->m);
    GPUNMF_CUDA_TRY(wh_residual_f32(j->n, j->m, j->r, j->W, j->H, j->V, j->red, s));
    GPUNMF_CUDA_TRY(finalize_partials(j->red, ctas, 2, 1, nullptr, S->d_res + q->slot, s));
    GPUNMF_CUDA_TRY(cudaMemcpyAsync(S->h_res + q->slot, S->d_res + q->slot, sizeof(double), cudaMemcpyDeviceToHost, s));
    return GPUNMF_OK;
}

// Capture a full chunk into a CUDA graph, so that each later chunk is one graph launch
// instead of some forty kernel launches from the scheduler thread.
static gpunmf_status capture_chunk(gpunmf_server *S, SJob *q) {
    cudaStream_t s = q->job->stream;
    cudaGraph_t g = nullptr;
    GPUNMF_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    gpunmf_status st = chunk_body(S, q, S->check_every);
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (st != GPUNMF_OK || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        if (st != GPUNMF_OK) return st;
        GPUNMF_CUDA_TRY(e);
    }
    e = cudaGraphInstantiate(&q->chunk_graph, g, 0);
    cudaGraphDestroy(g);
    GPUNMF_CUDA_TRY(e);
    return GPUNMF_OK;
}

static gpunmf_status enqueue_chunk(gpunmf_server *S, SJob *q) {
    gpunmf_job *j = q->job;
    const int chunk = std::min(S->check_every, S->max_iters - q->res.iters);
    if (chunk == S->check_every && q->chunk_graph) {
        GPUNMF_CUDA_TRY(cudaGraphLaunch(q->chunk_graph, j->stream));
    } else {
        gpunmf_status st = chunk_body(S, q, chunk);
        if (st != GPUNMF_OK) return st;
    }
    q->res.iters += chunk;
    GPUNMF_CUDA_TRY(cudaEventRecord(S->events[q->slot], j->stream));
    q->check_pending = true;
    return GPUNMF_OK;
}

static gpunmf_status start_job(gpunmf_server *S, SJob *q) {
    int prec = S->precision;
    if (prec == GPUNMF_BF16 && tc_supported(q->res.rule, q->res.n, q->res.m, q->res.r) != GPUNMF_OK)
        prec = GPUNMF_FP32;  // the tensor-core path does not cover this job: plain FP32
    q->res.precision = prec;
    int cap = 0;  // per-job CTA cap of the tensor-core kernels (0: every SM)
    const int bpc = S->blocks_per_cta.load();
    if (prec == GPUNMF_BF16 && bpc > 0) {
        const long long blocks = (long long)ceil_div(q->res.n, 128) * ceil_div(q->res.m, 128);
        cap = (int)std::min<long long>(std::max(1, S->max_job_ctas.load()), std::max<long long>(1, (blocks + bpc - 1) / bpc));
    }
    gpunmf_status st = job_create_empty(q->res.rule, q->res.n, q->res.m, q->res.r, q->eps, prec,
                                        S->streams[q->slot], S->h_pin + 64 * q->slot, true, &q->job, cap);
    if (st != GPUNMF_OK) return st;
    q->job->q_interval = 0;
    st = generate_job_data(q->job, q->seed, S->sigma);
    if (st == GPUNMF_OK) st = job_prepare(q->job);
    if (st == GPUNMF_OK && S->max_iters >= S->check_every) st = capture_chunk(S, q);
    if (st == GPUNMF_OK) st = enqueue_chunk(S, q);
    return st;
}

static void finish_job(gpunmf_server *S, SJob *q, int status) {
    if (q->chunk_graph) {
        cudaGraphExecDestroy(q->chunk_graph);
        q->chunk_graph = nullptr;
    }
    if (q->job) {
        if (S->keep && status == GPUNMF_OK) {
            q->W.resize((size_t)q->res.n * q->res.r);
            q->H.resize((size_t)q->res.r * q->res.m);
            cudaMemcpyAsync(q->W.data(), q->job->W, q->W.size() * 4, cudaMemcpyDeviceToHost, q->job->stream);
            cudaMemcpyAsync(q->H.data(), q->job->H, q->H.size() * 4, cudaMemcpyDeviceToHost, q->job->stream);
            cudaStreamSynchronize(q->job->stream);
        }
        job_release(q->job);
        q->job = nullptr;
    }
    q->res.status = status;
    q->res.t_done = S->now();
    std::lock_guard<std::mutex> lk(S->mu);
    if (q->slot >= 0) {
        S->slot_job[q->slot] = nullptr;
        S->free_slots.push_back(q->slot);
        S->in_use -= q->footprint;
    }
    q->slot = -1;
    S->done.push_back(q);
    S->finished++;
    S->cv_done.notify_all();
}

static void worker_loop(gpunmf_server *S) {
    cudaSetDevice(S->device);
    for (;;) {
        std::vector<SJob *> admitted;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            bool any_active = false;
            for (SJob *q : S->slot_job) any_active |= (q != nullptr);
            if (S->stop && S->pending.empty() && !any_active) break;
            while (!S->pending.empty() && !S->free_slots.empty()) {
                SJob *q = S->pending.front();
                if (q->footprint > S->budget) {  // can never fit: reject
                    S->pending.pop_front();
                    q->res.status = GPUNMF_ERR_REJECTED;
                    q->res.t_done = S->now();
                    S->done.push_back(q);
                    S->finished++;
                    S->cv_done.notify_all();
                    continue;
                }
                if (S->in_use + q->footprint > S->budget) break;  // wait for memory
                S->pending.pop_front();
                q->slot = S->free_slots.back();
                S->free_slots.pop_back();
                S->slot_job[q->slot] = q;
                S->in_use += q->footprint;
                q->res.t_admit = S->now();
                admitted.push_back(q);
            }
        }
        bool progress = !admitted.empty();
        for (SJob *q : admitted) {
            gpunmf_status st = start_job(S, q);
            if (st != GPUNMF_OK) finish_job(S, q, st);
        }
        for (size_t sl = 0; sl < S->slot_job.size(); sl++) {
            SJob *q;
            {
                std::lock_guard<std::mutex> lk(S->mu);
                q = S->slot_job[sl];
            }
            if (!q || !q->check_pending) continue;
            cudaError_t e = cudaEventQuery(S->events[sl]);
            if (e == cudaErrorNotReady) continue;
            progress = true;
            q->check_pending = false;
            if (e != cudaSuccess) {
                finish_job(S, q, GPUNMF_ERR_CUDA);
                continue;
            }
            q->res.residual = S->h_res[sl];
            if (q->res.residual <= S->tol || q->res.iters >= S->max_iters) {
                finish_job(S, q, GPUNMF_OK);
            } else {
                gpunmf_status st = enqueue_chunk(S, q);
                if (st != GPUNMF_OK) finish_job(S, q, st);
            }
        }
        if (!progress) {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv.wait_for(lk, std::chrono::microseconds(50));
        }
    }
}

extern "C" {

gpunmf_status gpunmf_server_create(int slots, size_t hbm_budget_bytes, int precision, int check_every, double tol,
                                   int max_iters, int keep_factors, gpunmf_server **out) {
    if (!out || slots <= 0 || slots > 1024 || check_every <= 0 || max_iters <= 0 ||
        (precision != GPUNMF_FP32 && precision != GPUNMF_BF16)) {
        set_error("invalid server arguments");
        return GPUNMF_ERR_INVALID;
    }
    int devs = 0;
    if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) {
        cudaGetLastError();
        set_error("no CUDA device available");
        return GPUNMF_ERR_NO_DEVICE;
    }
    gpunmf_server *S = new (std::nothrow) gpunmf_server();
    if (!S) return GPUNMF_ERR_NOMEM;
    S->slots = slots;
    S->budget = hbm_budget_bytes;
    S->precision = precision;
    S->check_every = check_every;
    S->tol = tol;
    S->max_iters = max_iters;
    S->keep = keep_factors != 0;
    S->t0 = std::chrono::steady_clock::now();
    cudaGetDevice(&S->device);
    S->streams.resize(slots);
    S->events.resize(slots);
    S->slot_job.assign(slots, nullptr);
    cudaError_t e = cudaSuccess;
    // keep freed blocks in the pool: retiring a job must not hand memory back to the driver
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, S->device) == cudaSuccess) {
        unsigned long long thr = ~0ULL;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    for (int k = 0; k < slots && e == cudaSuccess; k++) {
        e = cudaStreamCreateWithFlags(&S->streams[k], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S->events[k], cudaEventDisableTiming);
        S->free_slots.push_back(slots - 1 - k);
    }
    if (e == cudaSuccess) e = cudaMalloc((void **)&S->d_res, sizeof(double) * slots);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&S->h_res, sizeof(double) * slots, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&S->h_pin, 64 * (size_t)slots, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        set_error("server set-up failed: %s", cudaGetErrorString(e));
        cudaGetLastError();
        delete S;
        return GPUNMF_ERR_CUDA;
    }
    S->worker = std::thread(worker_loop, S);
    *out = S;
    return GPUNMF_OK;
}

gpunmf_status gpunmf_server_set_grid_policy(gpunmf_server *S, int blocks_per_cta, int max_job_ctas) {
    if (!S || blocks_per_cta < 0 || max_job_ctas < 0) {
        set_error("invalid grid policy");
        return GPUNMF_ERR_INVALID;
    }
    S->blocks_per_cta.store(blocks_per_cta);
    S->max_job_ctas.store(max_job_ctas > 0 ? max_job_ctas : kServeMaxJobCtas);
    return GPUNMF_OK;
}

gpunmf_status gpunmf_server_submit(gpunmf_server *S, long long id, int rule, int n, int m, int r,
                                   unsigned long long seed, float eps) {
    if (!S || n <= 0 || m <= 0 || r <= 0 || !rule_valid(rule)) {
        set_error("invalid job");
        return GPUNMF_ERR_INVALID;
    }
    SJob *q = new (std::nothrow) SJob();
    if (!q) return GPUNMF_ERR_NOMEM;
    q->res.id = id;
    q->res.rule = rule;
    q->res.n = n;
    q->res.m = m;
    q->res.r = r;
    q->res.residual = -1.0;
    q->seed = seed;
    q->eps = eps;
    int prec = S->precision;
    if (prec == GPUNMF_BF16 && tc_supported(rule, n, m, r) != GPUNMF_OK) prec = GPUNMF_FP32;
    q->footprint = job_footprint(rule, n, m, r, prec);
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) {
            delete q;
            set_error("server is draining");
            return GPUNMF_ERR_REJECTED;
        }
        q->res.t_submit = S->now();
        S->pending.push_back(q);
        S->submitted++;
    }
    S->cv.notify_one();
    return GPUNMF_OK;
}

// Copy up to `cap` finished results (oldest first) and forget them; returns how many.
int gpunmf_server_poll(gpunmf_server *S, gpunmf_server_result *out, int cap) {
    if (!S || !out || cap <= 0) return 0;
    std::lock_guard<std::mutex> lk(S->mu);
    int k = 0;
    while (k < cap && !S->done.empty()) {
        SJob *q = S->done.front();
        if (S->keep) break;  // keep mode: results are fetched with gpunmf_server_fetch
        S->done.erase(S->done.begin());
        out[k++] = q->res;
        delete q;
    }
    return k;
}

// keep_factors mode: result, W (n x r) and H (r x m) of a finished job by id (W/H may be NULL).
gpunmf_status gpunmf_server_fetch(gpunmf_server *S, long long id, gpunmf_server_result *res, float *W, float *H) {
    if (!S || !res) return GPUNMF_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    for (size_t k = 0; k < S->done.size(); k++) {
        SJob *q = S->done[k];
        if (q->res.id != id) continue;
        *res = q->res;
        if (W && !q->W.empty()) std::copy(q->W.begin(), q->W.end(), W);
        if (H && !q->H.empty()) std::copy(q->H.begin(), q->H.end(), H);
        return GPUNMF_OK;
    }
    set_error("job %lld is not finished", id);
    return GPUNMF_ERR_INVALID;
}

// Wait until every submitted job has finished or `timeout_s` passes; returns TIMEOUT in the latter case.
gpunmf_status gpunmf_server_drain(gpunmf_server *S, double timeout_s) {
    if (!S) return GPUNMF_ERR_INVALID;
    std::unique_lock<std::mutex> lk(S->mu);
    bool ok = S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                  [&] { return S->finished >= S->submitted; });
    return ok ? GPUNMF_OK : GPUNMF_ERR_TIMEOUT;
}

// Counters: submitted, finished, pending, active, bytes in use.
gpunmf_status gpunmf_server_stats(gpunmf_server *S, long long *submitted, long long *finished, int *pending,
                                  int *active, size_t *bytes_in_use) {
    if (!S) return GPUNMF_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    if (submitted) *submitted = S->submitted;
    if (finished) *finished = S->finished;
    if (pending) *pending = (int)S->pending.size();
    if (active) {
        int a = 0;
        for (SJob *q : S->slot_job) a += q != nullptr;
        *active = a;
    }
    if (bytes_in_use) *bytes_in_use = S->in_use;
    return GPUNMF_OK;
}

// Seconds since the server was created (the clock of the result timestamps).
double gpunmf_server_clock(gpunmf_server *S) { return S ? S->now() : -1.0; }

// Stop accepting jobs, cancel the pending ones (status REJECTED), finish the admitted ones, free everything.
gpunmf_status gpunmf_server_generate(int n, int m, int r, unsigned long long seed, float sigma, float *dV,
                                     float *dW, float *dH, void *stream) {
    if (n <= 0 || m <= 0 || r <= 0 || !dV || !dW || !dH || !(sigma >= 0.f)) {
        set_error("gpunmf_server_generate: invalid arguments");
        return GPUNMF_ERR_INVALID;
    }
    return generate_data(n, m, r, seed, sigma, dV, dW, dH, (cudaStream_t)stream);
}

gpunmf_status gpunmf_server_destroy(gpunmf_server *S) {
    if (!S) return GPUNMF_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        while (!S->pending.empty()) {
            SJob *q = S->pending.front();
            S->pending.pop_front();
            delete q;
        }
    }
    S->cv.notify_all();
    if (S->worker.joinable()) S->worker.join();
    for (SJob *q : S->done) delete q;
    for (int k = 0; k < S->slots; k++) {
        if (S->streams[k]) cudaStreamSynchronize(S->streams[k]);
        if (S->events[k]) cudaEventDestroy(S->events[k]);
        if (S->streams[k]) cudaStreamDestroy(S->streams[k]);
    }
    if (S->d_res) cudaFree(S->d_res);
    if (S->h_res) cudaFreeHost(S->h_res);
    if (S->h_pin) cudaFreeHost(S->h_pin);
    delete S;
    return GPUNMF_OK;
}

}  // extern "C"
