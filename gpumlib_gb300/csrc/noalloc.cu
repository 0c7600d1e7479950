// Relative-residual entry point that allocates no memory.
//
// gpunmf_residual_fp64 works on a job, and a job owns its workspaces (it
// allocates them when it is created).  Some callers cannot allocate at the
// point where they want a residual: a serving process whose device memory is
// all reserved up front by its own pool and admission budget (a stray
// cudaMalloc there can fail or overrun the budget, and cudaFree synchronises
// the whole device), or a convergence monitor running beside factorisations
// it does not own and only holds device pointers to.  For them this entry
// point takes the caller's device V, W, H and a device double for the result,
// and keeps its scratch -- one FP64 partial sum pair per CTA of the W*H
// product -- in a fixed array compiled into the library.
//
// Limits and sharing:
//  * the array holds kNoAllocMaxCtas pairs (1 MiB); a shape whose product
//    needs more CTAs is rejected with GPUNMF_ERR_INVALID;
//  * the array is a file-scope static __device__ variable, so every GPU that
//    loads the library holds it until the process exits;
//  * every call uses the same array and it keeps the last call's contents;
//    a call writes every partial it later reads, so nothing needs clearing,
//    but calls that overlap on the GPU (different streams, or threads) race
//    on it and must be serialised by the caller;
//  * the first call on each device looks the array's device address up with
//    cudaGetSymbolAddress (host code cannot use the array's name as a device
//    pointer); make that first call before any stream capture begins;
//  * the looked-up address is kept for the life of the process, so the entry
//    point must not be used on a device after cudaDeviceReset() on it (the
//    reset unloads the module and the kept address no longer names the array).
#include <mutex>

#include "common.cuh"
#include "kernels.h"

namespace {

constexpr int kNoAllocMaxCtas = 65536;
constexpr int kMaxDevices = 64;

std::mutex g_scratch_mu;
double *g_scratch_addr[kMaxDevices] = {};

}  // namespace

static __device__ __align__(256) double g_residual_scratch[2 * kNoAllocMaxCtas];

using namespace gpunmf;

extern "C" gpunmf_status gpunmf_residual_fp64_noalloc(int n, int m, int r, const float *dV, const float *dW,
                                                      const float *dH, double *dResult, void *stream) {
    if (n <= 0 || m <= 0 || r <= 0) {
        set_error("invalid shape n=%d m=%d r=%d", n, m, r);
        return GPUNMF_ERR_INVALID;
    }
    const int ctas = wh_reduce_ctas(n, m);
    if (ctas > kNoAllocMaxCtas) {
        set_error("gpunmf_residual_fp64_noalloc: n=%d x m=%d needs %d partial sums but the fixed scratch holds "
                  "%d; use gpunmf_residual_fp64 on a job for larger matrices",
                  n, m, ctas, kNoAllocMaxCtas);
        return GPUNMF_ERR_INVALID;
    }
    if (!dV || !dW || !dH || !dResult) {
        set_error("null device pointer");
        return GPUNMF_ERR_INVALID;
    }
    int dev = 0;
    GPUNMF_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("device ordinal %d out of range", dev);
        return GPUNMF_ERR_INVALID;
    }
    double *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        if (!g_scratch_addr[dev]) {
            double *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress((void **)&p, g_residual_scratch);
            if (e != cudaSuccess || !p) {
                set_error("cudaGetSymbolAddress of the residual scratch failed: %s", cudaGetErrorString(e));
                cudaGetLastError();
                return GPUNMF_ERR_CUDA;
            }
            g_scratch_addr[dev] = p;
        }
        scratch = g_scratch_addr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    GPUNMF_CUDA_TRY(wh_residual_f32(n, m, r, dW, dH, dV, scratch, s));
    GPUNMF_CUDA_TRY(finalize_partials(scratch, ctas, 2, 1, nullptr, dResult, s));
    return GPUNMF_OK;
}
