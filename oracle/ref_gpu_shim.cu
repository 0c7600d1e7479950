// C entry points around the reference's own GPU NMF classes, for the tests and the bench.
//
// TEST AND MEASUREMENT INFRASTRUCTURE ONLY.  oracle/build.py compiles this file
// together with the reference's sources for its GPU path, unchanged:
// src/algorithms/nmf/nmf_multiplicative_euclidian.cpp and
// nmf_multiplicative_divergence.cpp (the classes), src/cuda/nmf/nmf_kernels.cu
// and nmf_kernels_quality.cu (their kernels) and the headers they include
// (nmf_base.h, src/memory, src/common, src/cuda/definitions.h), with the
// definitions the reference's CMakeLists.txt:119-124 sets for compute
// capability >= 3.0, for sm_103a, linked against cuBLAS (DeviceMatrix.h
// multiplies through the legacy cublasSgemm).  The library that results
// (oracle/_ref/libref_gpu_nmf.so) is never part of the product: it is the
// reference arm's GPU implementation, timed beside the engine and compared with
// its FP32 path.
#include <chrono>
#include <cstring>

#include <cublas.h>
#include <cuda_runtime.h>

#include "algorithms/nmf/nmf_multiplicative_divergence.h"
#include "algorithms/nmf/nmf_multiplicative_euclidian.h"
#include "cuda/nmf/nmf_kernels.h"

using namespace GPUMLib;

namespace {

HostMatrix<cudafloat> host_matrix(int rows, int cols, const float *src) {
    HostMatrix<cudafloat> M(rows, cols, ColumnMajor);
    std::memcpy(M.Pointer(), src, sizeof(float) * (size_t)rows * cols);
    return M;
}

bool g_cublas = false;

}  // namespace

// cublasInit() as the reference's applications do before using DeviceMatrix::Multiply.
extern "C" int refgpu_init(void) {
    if (!g_cublas) g_cublas = (cublasInit() == CUBLAS_STATUS_SUCCESS);
    return g_cublas ? 0 : -1;
}

// rule 0: NMF_MultiplicativeEuclidianDistance, 1: NMF_MultiplicativeDivergence, built from
// V (n x m), W (n x r), H (r x m) column-major (the reference's (v, w, h) constructors,
// nmf_multiplicative_euclidian.h:62, nmf_multiplicative_divergence.h:51).  Runs `warmup`
// then `iters` calls of DoIteration(); W and H receive the factors after all of them.
// *seconds (nullable) gets the wall time of the `iters` calls, from a device
// synchronisation before the first to one after the last.  Returns 0, or a CUDA / cuBLAS
// error code (negative for cuBLAS).
template <class C>
int run(int n, int m, int r, const float *V, float *W, float *H, int warmup, int iters, double *seconds) {
    HostMatrix<cudafloat> v = host_matrix(n, m, V), w = host_matrix(n, r, W), h = host_matrix(r, m, H);
    C nmf(v, w, h);
    for (int i = 0; i < warmup; i++) nmf.DoIteration();
    cudaDeviceSynchronize();
    auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < iters; i++) nmf.DoIteration();
    cudaDeviceSynchronize();
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    int rc = (int)cudaGetLastError();
    if (rc == 0 && cublasGetError() != CUBLAS_STATUS_SUCCESS) rc = -3;
    HostMatrix<cudafloat> wo = nmf.GetW(), ho = nmf.GetH();
    std::memcpy(W, wo.Pointer(), sizeof(float) * (size_t)n * r);
    std::memcpy(H, ho.Pointer(), sizeof(float) * (size_t)r * m);
    return rc;
}

// The reference's block reductions (SumW, SumH, NMFquality in nmf_kernels.cu:63-233 and
// nmf_kernels_quality.cu:29-77) size their block as the power of two >= the count
// (NumberThreadsPerBlockThatBestFit) and finish with a warp step that reads sum[tid + 16]
// for every tid < 32: with 32 threads or fewer that reads past the block's shared
// allocation, an illegal address on this GPU.  So the shapes that give such a block are
// refused here (-4): the KL class with n <= 32 or m <= 32, any class with n * m <= 32, and
// the kernel wrappers below with blockSize < 64.
static bool reduction_blocks_ok(int rule, int n, int m) {
    if ((long long)n * m <= 32) return false;
    return rule != 1 || (n > 32 && m > 32);
}

extern "C" int refgpu_run(int rule, int n, int m, int r, const float *V, float *W, float *H, int warmup,
                          int iters, double *seconds) {
    if (refgpu_init() != 0) return -1;
    if (!reduction_blocks_ok(rule, n, m)) return -4;
    if (rule == 0) return run<NMF_MultiplicativeEuclidianDistance>(n, m, r, V, W, H, warmup, iters, seconds);
    if (rule == 1) return run<NMF_MultiplicativeDivergence>(n, m, r, V, W, H, warmup, iters, seconds);
    return -2;
}

// The reference's kernel-level functions that are C++ (namespace GPUMLib), under C names; the
// extern "C" ones (gpumlib_cuda_nmf_*, nmf_kernels.h:87-142) are exported by the library as they are.
// Device pointers; launches on the legacy default stream, as in the reference.  Return the
// launch's cudaError_t.
extern "C" int refgpu_kernel_quality(int blockSize, float *V, float *WH, int n, float *quality) {
    if (blockSize < 64) return -4;
    KernelNMFquality(blockSize, V, WH, n, quality);
    return (int)cudaGetLastError();
}

extern "C" int refgpu_kernel_sum_w(int blockSize, float *W, int n, int r, float *sumW) {
    if (blockSize < 64) return -4;
    KernelSumW(blockSize, W, n, r, sumW);
    return (int)cudaGetLastError();
}

extern "C" int refgpu_kernel_sum_h(int blockSize, float *H, int r, int m, float *sumH) {
    if (blockSize < 64) return -4;
    KernelSumH(blockSize, H, r, m, sumH);
    return (int)cudaGetLastError();
}
