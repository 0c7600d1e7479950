// Shared definitions for the GB300 NMF kernels and engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gpunmf.h"

namespace gpunmf {

// Reference epsilon SMALL_VALUE_TO_ADD_DENOMINATOR = 10e-9 (src/cuda/nmf/nmf_kernels.h:34).
constexpr float kReferenceEps = 1e-8f;

constexpr int kNumSMsGB300 = 152;

// Set by the engine; the error text of the last failure on this thread.
void set_error(const char *fmt, ...);

#define GPUNMF_CUDA_TRY(expr)                                                           \
    do {                                                                                \
        cudaError_t _e = (expr);                                                        \
        if (_e != cudaSuccess) {                                                        \
            ::gpunmf::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                                __FILE__, __LINE__);                                    \
            return _e == cudaErrorMemoryAllocation ? GPUNMF_ERR_NOMEM : GPUNMF_ERR_CUDA; \
        }                                                                               \
    } while (0)

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of a double; every thread gets the result.  blockDim.x must be
// a multiple of 32 and at most 1024.  `red` needs 32 doubles of shared memory.
__device__ __forceinline__ double block_sum(double v, double *red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double t = (threadIdx.x < nw) ? red[threadIdx.x] : 0.0;
    if (wid == 0) t = warp_sum(t);
    if (threadIdx.x == 0) red[0] = t;
    __syncthreads();
    double out = red[0];
    __syncthreads();
    return out;
}

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace gpunmf
