/*
 * gpunmf.h — C ABI of the GB300 multiplicative-update NMF engine.
 *
 * Plain C: pointers, sizes and status codes only.  Every matrix at this
 * boundary is FP32 and column-major, exactly as GPUMLib requires of its
 * callers (src/algorithms/nmf/nmf_base.h:92,109-114):
 *   V  n x m   (element (i,u) at V[u*n + i])
 *   W  n x r   (element (i,a) at W[a*n + i])
 *   H  r x m   (element (a,u) at H[u*r + a])
 *
 * Two layers are exported:
 *
 *  1. Job API (gpunmf_*): what GPUMLib's NMF classes do
 *     (src/algorithms/nmf/nmf_base.h:45-151,
 *      nmf_multiplicative_euclidian.{h,cpp}, nmf_multiplicative_divergence.{h,cpp}),
 *     as an opaque handle that owns the device copies of V, W and H.
 *     include/gpumlib_nmf.hpp wraps it in the reference's C++ classes.
 *
 *  2. Kernel API (gpumlib_cuda_nmf_*, gpumlib_nmf_*): the reference's
 *     extern "C" launch wrappers of src/cuda/nmf/nmf_kernels.h:87,100,113 with
 *     the same names and arguments, plus C entry points for its C++-linkage
 *     helpers KernelSumW / KernelSumH / KernelNMFquality
 *     (nmf_kernels.h:44,64,73).  They take device pointers, launch on the
 *     legacy default stream like the reference, and return the launch's
 *     cudaError_t (as int).
 *
 * Status codes: every gpunmf_* call returns gpunmf_status.  Nothing is
 * printed and nothing aborts; a CUDA failure is reported as GPUNMF_ERR_CUDA
 * and its text is kept for gpunmf_last_error().
 */
#ifndef GPUNMF_H
#define GPUNMF_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GPUNMF_OK = 0,
    GPUNMF_ERR_INVALID = 1,      /* bad handle, shape, pointer or option  */
    GPUNMF_ERR_CUDA = 2,         /* a CUDA call failed (see last_error)   */
    GPUNMF_ERR_NOMEM = 3,        /* device or pinned allocation failed    */
    GPUNMF_ERR_UNSUPPORTED = 4,  /* option not available for this job     */
    GPUNMF_ERR_NO_DEVICE = 5,    /* no CUDA device, or not an sm_103 GPU   */
    GPUNMF_ERR_TIMEOUT = 6,      /* a bounded device wait gave up         */
    GPUNMF_ERR_REJECTED = 7      /* admission control refused a job       */
} gpunmf_status;

/* Update rules (GPUMLib class names in brackets). */
typedef enum {
    GPUNMF_EUCLIDEAN = 0,            /* NMF_MultiplicativeEuclidianDistance              */
    GPUNMF_DIVERGENCE = 1,           /* NMF_MultiplicativeDivergence (KL)                */
    GPUNMF_ADDITIVE_EUCLIDEAN = 2,   /* additive Euclidean rule with both factors updated
                                        (HostNMF::DoIteration_AE, HostNMF.h:152-190)      */
    GPUNMF_ADDITIVE_DIVERGENCE = 3,  /* NMF_AdditiveDivergence (additive KL)             */
    GPUNMF_ADDITIVE_EUCLIDEAN_FIXED_H = 4
                                     /* NMF_AdditiveEuclidian exactly as the reference's GPU
                                        class runs it: its H step hands (H, deltaH, deltaH2)
                                        to the multiplicative kernel, which overwrites the
                                        deltaH2 workspace, so H keeps its initial value
                                        (nmf_additive_euclidian.cpp:37-42)                */
} gpunmf_rule;

/* Arithmetic of the factor products.  The W/H update itself is always FP32. */
typedef enum {
    GPUNMF_FP32 = 0,        /* plain FP32 (CUDA cores): the drop-in path         */
    GPUNMF_BF16 = 1         /* BF16 tensor-core products (tcgen05), FP32 accumulate */
} gpunmf_precision;

typedef struct gpunmf_job *gpunmf_handle;

/* Reference epsilon: SMALL_VALUE_TO_ADD_DENOMINATOR = 10e-9 (nmf_kernels.h:34). */
#define GPUNMF_REFERENCE_EPS 1e-8f

/* Text of the last error on this thread ("" if none). */
const char *gpunmf_last_error(void);

/* Library version string. */
const char *gpunmf_version(void);

/* Number of CUDA devices visible (0 when none). */
int gpunmf_device_count(void);

/*
 * Create a job from HOST matrices (copied to the device), like
 * NMF(v, w, h) (nmf_base.h:108-120).  W and H are the initial factors.
 * stream: a cudaStream_t (NULL = the library creates its own stream).
 * eps: denominator guard; GPUNMF_REFERENCE_EPS reproduces the reference.
 */
gpunmf_status gpunmf_create(int rule, int n, int m, int r,
                            const float *V, const float *W, const float *H,
                            float eps, int precision, void *stream,
                            gpunmf_handle *out);

/*
 * Create a job like NMF(v, r) (nmf_base.h:91-106): W and H are drawn on the
 * host as uniform[0,1) + eps from a counter-based generator keyed by seed
 * (the reference draws them from an unseeded rand()).
 */
gpunmf_status gpunmf_create_random(int rule, int n, int m, int r, const float *V,
                                   unsigned long long seed, float eps, int precision,
                                   void *stream, gpunmf_handle *out);

/* Same as gpunmf_create but V, W, H are DEVICE pointers (copied on the job's stream). */
gpunmf_status gpunmf_create_device(int rule, int n, int m, int r,
                                   const float *dV, const float *dW, const float *dH,
                                   float eps, int precision, void *stream,
                                   gpunmf_handle *out);

gpunmf_status gpunmf_destroy(gpunmf_handle h);

/*
 * Run `iters` iterations of DoIteration(updateW) (nmf_base.h:145).
 * Order per iteration: H first, then (if updateW) W with the new H.
 * Enqueued on the job's stream; returns without waiting for the GPU.
 */
gpunmf_status gpunmf_iterate(gpunmf_handle h, int iters, int updateW);

/*
 * Quality bookkeeping of DetermineQualityImprovement (nmf_base.h:70-89).
 * interval k > 0: the log10 quality is evaluated every k-th iteration, and
 * each sample first waits for the previous one's read-back (deterministic:
 * 1 = every iteration, the reference's behaviour when its GPU keeps up);
 * 0 turns it off; GPUNMF_QUALITY_WHEN_READY is the reference's own rule:
 * an iteration samples only if the previous sample's read-back has completed
 * (nmf_base.h:71 queries the read-back's stream), never waiting for it, so
 * which iterations sample depends on how far the host runs ahead of the GPU.
 * Default: 1.
 */
#define GPUNMF_QUALITY_WHEN_READY (-1)
gpunmf_status gpunmf_set_quality_interval(gpunmf_handle h, int interval);

/*
 * Bounded device waits (no counterpart in the reference, whose kernels never
 * wait on one another).  The BF16 kernels' CTAs wait on one another (tile
 * arrivals, grid-wide sums); every such wait gives up after a limit of SM
 * clock cycles, sets the job's error word, and the next call that reads it
 * (synchronize, get, residual) returns GPUNMF_ERR_TIMEOUT; the job must then be
 * destroyed.  Default limit: 4e9 cycles (about 2 s at 2 GHz); cycles <= 0
 * restores it.  Applies to the job's later launches.  BF16 jobs only.
 */
gpunmf_status gpunmf_set_wait_limit_cycles(gpunmf_handle h, long long cycles);

/*
 * Host-side fault injection for tests of the path above: the arrival counter
 * of the first row tile of the job's next fused half-step starts one below
 * zero, so the fused update's wait for that tile cannot complete and runs out
 * (bounded).  No GPU fault: the kernel returns with its error word set.
 * GPUNMF_ERR_UNSUPPORTED for jobs without a fused update.
 */
gpunmf_status gpunmf_inject_missing_arrival(gpunmf_handle h);

/*
 * CTAs per launch of the tensor-core kernels of jobs created after this call
 * (0 = one per SM, the default).  The fused kernels need their whole grid
 * resident at once; an application that keeps long-running kernels of its own
 * on some SMs (persistent kernels of another library, on other streams) caps
 * the grid below the SMs those leave free, so the fused grid never waits for
 * SMs that do not come free.  Process-wide.
 */
gpunmf_status gpunmf_set_grid_limit(int ctas);

/* QualityImprovement() (nmf_base.h:148-150): lagged change of the quality; 1.0 initially. */
gpunmf_status gpunmf_quality_improvement(gpunmf_handle h, float *out);

/* Relative Frobenius residual ||V - W H||_F / ||V||_F of the current factors,
 * WH in FP32 from the FP32 factors, squares accumulated in FP64 on the GPU. */
gpunmf_status gpunmf_residual_fp64(gpunmf_handle h, double *out);

/*
 * Allocation-free relative residual (no counterpart in the reference).
 * ||V - W H||_F / ||V||_F of caller-owned DEVICE matrices (column-major FP32),
 * computed like gpunmf_residual_fp64 and written to the DEVICE double
 * *dResult on `stream` (NULL = legacy default stream); returns without
 * waiting.  For callers that must not allocate device memory at this point
 * (a process whose memory is all reserved by its own pool, or a monitor that
 * only holds device pointers to someone else's factors): its scratch is a
 * fixed 1 MiB array inside the library, one FP64 pair per CTA of the W*H
 * product, at most 65536 CTAs; larger shapes are rejected with
 * GPUNMF_ERR_INVALID.  All calls share that array: calls that overlap on the
 * GPU race.  The first call on each device looks up the array's address;
 * make it before any stream capture begins.  The address is kept for the
 * life of the process: do not call this on a device after cudaDeviceReset()
 * on that device.
 */
gpunmf_status gpunmf_residual_fp64_noalloc(int n, int m, int r, const float *dV, const float *dW,
                                           const float *dH, double *dResult, void *stream);

/* Generalised KL objective sum V log(V/WH) - V + WH (FP64 on the GPU). */
gpunmf_status gpunmf_objective_kl_fp64(gpunmf_handle h, double *out);

/* GetW / GetH / GetWH (nmf_base.h:125-141): synchronous copies to host
 * buffers of n*r, r*m and n*m floats, column-major. */
gpunmf_status gpunmf_get_w(gpunmf_handle h, float *W);
gpunmf_status gpunmf_get_h(gpunmf_handle h, float *H);
gpunmf_status gpunmf_get_wh(gpunmf_handle h, float *WH);

/* Device pointers of the job's FP32 factors (valid until destroy). */
gpunmf_status gpunmf_device_factors(gpunmf_handle h, float **dW, float **dH);

/* Wait for the job's queued work. */
gpunmf_status gpunmf_synchronize(gpunmf_handle h);

/* Shape/options of a job. */
gpunmf_status gpunmf_info(gpunmf_handle h, int *rule, int *n, int *m, int *r,
                          int *precision, float *eps);

/* Device bytes a job of this shape holds (admission accounting). */
size_t gpunmf_footprint_bytes(int rule, int n, int m, int r, int precision);

/* Jobs made through this API take device memory from a pool the library keeps per device, so
 * creating a job after another was destroyed needs no driver allocation.  This hands the pool's
 * unused memory back to the driver (for the current device); jobs still alive keep theirs. */
gpunmf_status gpunmf_trim_pool(void);

/* Host-only: out[k] = uniform[0,1) value number offset+k of the counter-based
 * generator keyed by seed (the generator gpunmf_create_random uses). */
void gpunmf_fill_uniform(unsigned long long seed, unsigned long long offset, size_t count, float *out);

/* Page-locked host buffers for end-to-end transfers (NULL on failure). */
void *gpunmf_host_alloc(size_t bytes);
void gpunmf_host_free(void *p);

/*
 * Timing helper: enqueue `iters` iterations bracketed by CUDA events on the
 * job's stream, wait, and return the elapsed milliseconds.  When
 * kernel_ms/kernel_launches are given, the two V-streaming kernels of each
 * iteration are also bracketed by events and their summed device time and
 * launch count are returned (for the roofline of the dominant kernel).
 */
gpunmf_status gpunmf_time_iterations(gpunmf_handle h, int iters, int updateW,
                                     float *total_ms, float *kernel_ms,
                                     int *kernel_launches, int *all_launches);

/* ------------------------------------------------------------------ */
/* Batched small factorisations (Euclidean rule, FP32, ranks 1..32):   */
/* the counterpart of FacesNMF's grouped training, which runs one NMF  */
/* object per group in turn (src/examples/FacesNMF/FacesNMFDlg.cpp:    */
/* 582-656).  All instances run in one persistent, graph-captured      */
/* launch; each CTA takes whole instances, largest first.              */
/* ------------------------------------------------------------------ */
typedef struct gpunmf_batch gpunmf_batch;

/* Instances k < count: V[k] n[k] x m[k], W[k] n[k] x r[k], H[k] r[k] x m[k] (host, column-major). */
gpunmf_status gpunmf_batch_create(int count, const int *n, const int *m, const int *r, const float *const *V,
                                  const float *const *W, const float *const *H, float eps,
                                  gpunmf_batch **out);
gpunmf_status gpunmf_batch_destroy(gpunmf_batch *b);
/* `iters` iterations of every instance; enqueued, returns without waiting. */
gpunmf_status gpunmf_batch_run(gpunmf_batch *b, int iters);
gpunmf_status gpunmf_batch_synchronize(gpunmf_batch *b);
/* Device time (CUDA events) of one gpunmf_batch_run(b, iters), milliseconds. */
gpunmf_status gpunmf_batch_time(gpunmf_batch *b, int iters, float *ms);
/* Copy instance k's W (n x r) and/or H (r x m) to host buffers (NULL to skip). */
gpunmf_status gpunmf_batch_get(gpunmf_batch *b, int k, float *W, float *H);
/* Relative Frobenius residual of every instance (count doubles), FP64 on the GPU. */
gpunmf_status gpunmf_batch_residuals(gpunmf_batch *b, double *out);
/* Tile configurations: returns their number; ranks[c] = rank class (4, 8, 16, 32) of config c. */
int gpunmf_batch_configs(int *ranks, int cap);
/* Choose instance k's tile configuration (same rank class), then commit before running. */
gpunmf_status gpunmf_batch_set_config(gpunmf_batch *b, int k, int cfg);
gpunmf_status gpunmf_batch_commit(gpunmf_batch *b);
/* Overwrite every instance's W and H from host buffers (same shapes as at creation). */
gpunmf_status gpunmf_batch_reset_factors(gpunmf_batch *b, const float *const *W, const float *const *H);

/* Grouped training, FacesNMFDlg.cpp:582-656 (TrainUsingGroups).  Host, column-major V (n x m),
 * W (n x r) and H (r x m); W and H are inputs and outputs.  The first blocks = floor(m/group)
 * blocks of `group` consecutive columns of V are factorised independently with rank
 * rs = floor(r/blocks), block s starting from W's columns s*rs.. and the diagonal block of H (rows
 * s*rs.., columns s*group..) -- the reference starts each block from fresh rand() factors.  Each
 * block iterates its rule until QualityImprovement() changes to a value below tol, the
 * reference's test, or max_iters.  Results: W's columns s*rs.. and, in the block's columns of H,
 * the block's H in rows s*rs.. and zeros elsewhere; W columns from blocks*rs and H columns from
 * blocks*group are returned unchanged.  iterations (nullable) receives `blocks` counts.
 * The multiplicative Euclidean rule in FP32 with rs <= 32 runs all blocks in one persistent
 * batched launch; other rules and precisions run one job per block, many at a time. */
gpunmf_status gpunmf_grouped_train(int rule, int n, int m, int r, int group, const float *V, float *W,
                                   float *H, float tol, int max_iters, float eps, int precision,
                                   int *iterations);

/* ------------------------------------------------------------------ */
/* FacesNMF data set I/O (src/examples/FacesNMF/FacesNMFDlg.cpp).       */
/* ------------------------------------------------------------------ */
/* FolderHasImages (:309-347): reads folder/face00001.pgm's P5 header for the image size and counts
 * the images face00001.pgm.. by the reference's probe (steps of 1024, halved on every miss). */
gpunmf_status gpunmf_faces_scan(const char *folder, int *count, int *width, int *height);

/* LoadImage (:409-472) for images 1..count into V (width*height x count, column-major FP32), host
 * (gpunmf_faces_load) or device memory (gpunmf_faces_load_device, on `stream`, NULL = a private one).
 * equalize: the reference's histogram equalisation; else pixel / 255.  reference_offset = 1 reads the
 * pixel block where the reference does, starting at the whitespace byte that ends the header (pixel 0
 * is that byte, the last pixel is not read); 0 reads it where the PGM format puts it.  Images that
 * fail (format, size, max gray value other than 255, short file) get a zero column, the others are
 * loaded, and the call returns GPUNMF_ERR_INVALID with *failed (nullable) = how many failed. */
gpunmf_status gpunmf_faces_load(const char *folder, int count, int width, int height, int equalize,
                                int reference_offset, float *V, int *failed);
gpunmf_status gpunmf_faces_load_device(const char *folder, int count, int width, int height, int equalize,
                                       int reference_offset, float *dV, void *stream, int *failed);

/* Save (:913-924): one line per COLUMN of the rows x cols column-major matrix, its values
 * comma-separated in fixed notation with 20 decimals (PRECISION, Definitions.h:31), '\n' after each
 * line.  _device: the matrix is in device memory (read back on `stream`). */
gpunmf_status gpunmf_save_csv(const char *path, const float *M, int rows, int cols);
gpunmf_status gpunmf_save_csv_device(const char *path, const float *dM, int rows, int cols, void *stream);

/* ------------------------------------------------------------------ */
/* Serving with continuous batching.  Jobs arrive at any time; a       */
/* scheduler thread admits each one as soon as one of `slots` stream   */
/* slots is free and its device footprint fits `hbm_budget_bytes`,     */
/* advances every admitted job in chunks of `check_every` iterations,  */
/* each followed by an FP64 relative-residual check, and retires a job */
/* at residual <= tol or max_iters iterations.  Admitted jobs' kernels  */
/* overlap on the device.  Job data (V = A B + |N(0,0.01)|, W, H) is    */
/* generated on the device from the job's seed.                        */
/* ------------------------------------------------------------------ */
typedef struct gpunmf_server gpunmf_server;

typedef struct {
    long long id;
    int rule, n, m, r, iters, precision, status;   /* status: gpunmf_status of the job */
    double residual, t_submit, t_admit, t_done;     /* seconds on the server clock */
} gpunmf_server_result;

/* keep_factors != 0 keeps each finished job's W and H on the host for gpunmf_server_fetch
 * (then gpunmf_server_poll returns nothing). */
gpunmf_status gpunmf_server_create(int slots, size_t hbm_budget_bytes, int precision, int check_every,
                                   double tol, int max_iters, int keep_factors, gpunmf_server **out);
gpunmf_status gpunmf_server_submit(gpunmf_server *s, long long id, int rule, int n, int m, int r,
                                   unsigned long long seed, float eps);
/* CTAs per launch of each admitted BF16 job's tensor-core kernels: ceil(blocks / blocks_per_cta),
 * at least 1 and at most max_job_ctas, where blocks = ceil(n/128) ceil(m/128).  Capping the large
 * jobs' grids lets more jobs share the SMs at once.  blocks_per_cta 0: every job may use every SM
 * (as a job created alone does); max_job_ctas 0: the default cap.  Applies to jobs admitted after
 * the call.  Defaults: 1 block per CTA, at most 24 CTAs. */
gpunmf_status gpunmf_server_set_grid_policy(gpunmf_server *s, int blocks_per_cta, int max_job_ctas);
/* Move up to `cap` finished results into out[]; returns their number. */
int gpunmf_server_poll(gpunmf_server *s, gpunmf_server_result *out, int cap);
gpunmf_status gpunmf_server_fetch(gpunmf_server *s, long long id, gpunmf_server_result *res, float *W, float *H);
/* Wait for every submitted job (GPUNMF_ERR_TIMEOUT after timeout_s seconds). */
gpunmf_status gpunmf_server_drain(gpunmf_server *s, double timeout_s);
gpunmf_status gpunmf_server_stats(gpunmf_server *s, long long *submitted, long long *finished, int *pending,
                                  int *active, size_t *bytes_in_use);
double gpunmf_server_clock(gpunmf_server *s);
/* Cancels pending jobs, finishes admitted ones, frees everything. */
gpunmf_status gpunmf_server_destroy(gpunmf_server *s);
/* The data a served job with this seed starts from, written by the same device code into caller
 * DEVICE buffers (V n x m, W n x r, H r x m; sigma 0.01 as the server uses), on `stream`: lets a
 * caller rebuild a served job's inputs, e.g. to check its result against another implementation. */
gpunmf_status gpunmf_server_generate(int n, int m, int r, unsigned long long seed, float sigma, float *dV,
                                     float *dW, float *dH, void *stream);

/* ------------------------------------------------------------------ */
/* Kernel API: same names and arguments as src/cuda/nmf/nmf_kernels.h. */
/* gridDim/blockDim are accepted for source compatibility; the GB300   */
/* kernels pick their own launch shape (vectorised, grid-stride).      */
/* Return value: cudaError_t of the launch (0 = cudaSuccess).          */
/* ------------------------------------------------------------------ */
typedef struct { unsigned int x, y, z; } gpunmf_dim3;   /* layout of CUDA's dim3 */

/* nmf_kernels.h:87 — m[i] *= nm[i] / (dm[i] + 1e-8), i < elements */
int gpumlib_cuda_nmf_multiplicative_euclidean_update_matrix(
    unsigned int gridDim, unsigned int blockDim, float *nm, float *dm, float *m, int elements);

/* nmf_kernels.h:100 — W(i,a) *= [sum_u H(a,u) V(i,u)/(WH(i,u)+1e-8)] / sumH[a] */
int gpumlib_cuda_nmf_multiplicative_divergence_update_matrix_w(
    gpunmf_dim3 gridDim, gpunmf_dim3 blockDim, float *W, float *H, float *V, float *WH,
    float *sumH, int n, int m, int r);

/* nmf_kernels.h:113 — H(a,u) *= [sum_i W(i,a) V(i,u)/(WH(i,u)+1e-8)] / sumW[a] */
int gpumlib_cuda_nmf_multiplicative_divergence_update_matrix_h(
    gpunmf_dim3 gridDim, gpunmf_dim3 blockDim, float *H, float *W, float *V, float *WH,
    float *sumW, int n, int m, int r);

/* nmf_kernels.h:116 — X[i] = max(0, X[i] + (X[i] / deltaX2[i]) * (deltaX1[i] - deltaX2[i])) */
int gpumlib_cuda_nmf_additive_euclidean_update_matrix(
    unsigned int gridDim, unsigned int blockDim, float *X, float *deltaX1, float *deltaX2, int elements);

/* nmf_kernels.h:142 —
   W(i,a) = max(0, W + (W / sumH[a]) * sum_u H(a,u) [V(i,u)/(WH(i,u)+1e-8) - 1]) */
int gpumlib_cuda_nmf_additive_divergence_update_matrix_w(
    gpunmf_dim3 gridDim, gpunmf_dim3 blockDim, float *W, float *H, float *V, float *WH,
    float *sumH, int n, int m, int r);

/* nmf_kernels.h:129 —
   H(a,u) = max(0, H + (H / sumW[a]) * sum_i W(i,a) [V(i,u)/(WH(i,u)+1e-8) - 1]) */
int gpumlib_cuda_nmf_additive_divergence_update_matrix_h(
    gpunmf_dim3 gridDim, gpunmf_dim3 blockDim, float *H, float *W, float *V, float *WH,
    float *sumW, int n, int m, int r);

/* nmf_kernels.h:64 (KernelSumW) — sumW[a] = max(sum_i W(i,a), 1e-8) */
int gpumlib_nmf_sum_w(int blockSize, float *W, int n, int r, float *sumW);

/* nmf_kernels.h:73 (KernelSumH) — sumH[a] = max(sum_u H(a,u), 1e-8) */
int gpumlib_nmf_sum_h(int blockSize, float *H, int r, int m, float *sumH);

/* nmf_kernels.h:44 (KernelNMFquality) — *quality = sum_k V[k] log10(WH[k]+1e-8) - WH[k] */
int gpumlib_nmf_quality(int blockSize, float *V, float *WH, int n, float *quality);

#ifdef __cplusplus
}
#endif

#endif /* GPUNMF_H */
