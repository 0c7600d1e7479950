// Kernel-level entry points with the reference's names and arguments
// (src/cuda/nmf/nmf_kernels.h:44,64,73,87,100,113,116,129,142).  Like the reference they
// launch on the legacy default stream and return the launch's cudaError_t;
// the grid/block arguments are accepted for source compatibility, and the
// launch shape is chosen here (vectorised grid-stride elementwise kernel,
// tiled products, warp-shuffle reductions).
#include "common.cuh"
#include "kernels.h"

using namespace gpunmf;

namespace {
__global__ void mu_update_kernel(const float *__restrict__ nm, const float *__restrict__ dm, float *__restrict__ x,
                                 long long count) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count; k += stride)
        x[k] *= nm[k] / (dm[k] + kReferenceEps);
}

__global__ void additive_euclid_kernel(const float *__restrict__ d1, const float *__restrict__ d2,
                                       float *__restrict__ x, long long count) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count; k += stride) {
        float xv = x[k], d = d2[k];
        float v = xv + (xv / d) * (d1[k] - d);
        x[k] = v < 0.0f ? 0.0f : v;
    }
}

__global__ void quality_single_kernel(const double *partial, int count, float *quality) {
    __shared__ double red[32];
    double s = 0.0;
    for (int c = threadIdx.x; c < count; c += blockDim.x) s += partial[c];
    s = block_sum(s, red);
    if (threadIdx.x == 0) *quality = (float)s;
}

// FP64 partials for gpumlib_nmf_quality: kept in device memory owned by the
// library (grown on demand, freed at exit by the driver).
double *g_quality_partials = nullptr;
int g_quality_cap = 0;
}  // namespace

extern "C" {

int gpumlib_cuda_nmf_multiplicative_euclidean_update_matrix(unsigned int, unsigned int, float *nm, float *dm,
                                                            float *m, int elements) {
    if (elements <= 0) return (int)cudaSuccess;
    long long blocks = (elements + 255) / 256;
    if (blocks > 8 * kNumSMsGB300) blocks = 8 * kNumSMsGB300;
    mu_update_kernel<<<(int)blocks, 256>>>(nm, dm, m, elements);
    return (int)cudaGetLastError();
}

int gpumlib_cuda_nmf_additive_euclidean_update_matrix(unsigned int, unsigned int, float *X, float *deltaX1,
                                                      float *deltaX2, int elements) {
    if (elements <= 0) return (int)cudaSuccess;
    long long blocks = (elements + 255) / 256;
    if (blocks > 8 * kNumSMsGB300) blocks = 8 * kNumSMsGB300;
    additive_euclid_kernel<<<(int)blocks, 256>>>(deltaX1, deltaX2, X, elements);
    return (int)cudaGetLastError();
}

int gpumlib_cuda_nmf_additive_divergence_update_matrix_w(gpunmf_dim3, gpunmf_dim3, float *W, float *H, float *V,
                                                         float *WH, float *sumH, int n, int m, int r) {
    return (int)akl_update_w_ref(W, H, V, WH, sumH, n, m, r, kReferenceEps, 0);
}

int gpumlib_cuda_nmf_additive_divergence_update_matrix_h(gpunmf_dim3, gpunmf_dim3, float *H, float *W, float *V,
                                                         float *WH, float *sumW, int n, int m, int r) {
    return (int)akl_update_h_ref(H, W, V, WH, sumW, n, m, r, kReferenceEps, 0);
}

int gpumlib_cuda_nmf_multiplicative_divergence_update_matrix_w(gpunmf_dim3, gpunmf_dim3, float *W, float *H,
                                                               float *V, float *WH, float *sumH, int n, int m,
                                                               int r) {
    return (int)kl_update_w_ref(W, H, V, WH, sumH, n, m, r, kReferenceEps, 0);
}

int gpumlib_cuda_nmf_multiplicative_divergence_update_matrix_h(gpunmf_dim3, gpunmf_dim3, float *H, float *W,
                                                               float *V, float *WH, float *sumW, int n, int m,
                                                               int r) {
    return (int)kl_update_h_ref(H, W, V, WH, sumW, n, m, r, kReferenceEps, 0);
}

int gpumlib_nmf_sum_w(int, float *W, int n, int r, float *sumW) {
    return (int)col_sums(W, n, r, kReferenceEps, sumW, 0);
}

int gpumlib_nmf_sum_h(int, float *H, int r, int m, float *sumH) {
    return (int)row_sums(H, r, m, kReferenceEps, sumH, 0);
}

int gpumlib_nmf_quality(int, float *V, float *WH, int n, float *quality) {
    int ctas = quality_ew_ctas(n);
    if (ctas > g_quality_cap) {
        if (g_quality_partials) cudaFree(g_quality_partials);
        g_quality_partials = nullptr;
        g_quality_cap = 0;
        cudaError_t e = cudaMalloc((void **)&g_quality_partials, sizeof(double) * ctas);
        if (e != cudaSuccess) return (int)e;
        g_quality_cap = ctas;
    }
    cudaError_t e = quality_ew(V, WH, n, kReferenceEps, g_quality_partials, 0);
    if (e != cudaSuccess) return (int)e;
    quality_single_kernel<<<1, 512>>>(g_quality_partials, ctas, quality);
    return (int)cudaGetLastError();
}

}  // extern "C"
