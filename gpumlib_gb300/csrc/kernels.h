// Internal launcher declarations shared by the engine and the kernel files.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace gpunmf {

// ---------------- FP32 CUDA-core products (f32_kernels.cu) ----------------
// Column-major operands.  op(A) is M x K, op(B) is K x N; the *_t flags say
// the stored matrix is the transpose of the operand.  `splits` > 1 writes
// split-K partial products: P[z*M*N + j*M + i] (column-major, ld = M).
struct F32Operand {
    const float *p;
    long long ld;
    bool t;
};

// C = op(A) op(B) (splits == 1: straight into C with ldc; else into partials P).
cudaError_t gemm_f32(int M, int N, int K, F32Operand A, F32Operand B, float *C, long long ldc,
                     int splits, cudaStream_t s);

// C = R op(B) (left) or op(A) R (right) where R = V / (WH + eps) is formed while loading
// (the KL ratio, src/cuda/nmf/nmf_kernels.cu:271,319); minus_one forms V / (WH + eps) - 1
// instead (the additive KL rule, src/cuda/nmf/nmf_kernels_additive_divergence.cu:90,159).
cudaError_t gemm_f32_ratio_left(int M, int N, int K, const float *V, const float *WH, long long ldv,
                                float eps, F32Operand B, float *P, int splits, cudaStream_t s,
                                bool minus_one = false);
cudaError_t gemm_f32_ratio_right(int M, int N, int K, F32Operand A, const float *V, const float *WH,
                                 long long ldv, float eps, float *P, int splits, cudaStream_t s,
                                 bool minus_one = false);

// Number of split-K slices gemm_f32* will use for this shape (so callers can size partials).
int gemm_f32_splits(int M, int N, int K);
// Number of CTAs of the reducing product kernels below (for partial buffers).
int wh_reduce_ctas(int n, int m);

// Fused W*H product with a reduction epilogue: never stores WH.
//  quality:  partial[cta] = sum V*log10(WH+eps) - WH            (nmf_kernels_quality.cu:35)
//  residual: partial[2*cta] = sum (V-WH)^2, partial[2*cta+1] = sum V^2
cudaError_t wh_quality_f32(int n, int m, int r, const float *W, const float *H, const float *V,
                           float eps, double *partial, cudaStream_t s);
cudaError_t wh_residual_f32(int n, int m, int r, const float *W, const float *H, const float *V,
                            double *partial, cudaStream_t s);

// Elementwise quality over a stored WH (KL path).  partial needs quality_ew_ctas() doubles.
int quality_ew_ctas(long long count);
cudaError_t quality_ew(const float *V, const float *WH, long long count, float eps, double *partial,
                       cudaStream_t s);
// KL objective sum V log(V/WH) - V + WH over a stored WH (FP64 accumulation).
cudaError_t kl_objective_ew(const float *V, const float *WH, long long count, double *partial,
                            cudaStream_t s);

// Sum `count` partials (stride `terms`) in a fixed order.  mode 0: out_f[0] = (float)sum0,
// out_d[0] = sum0.  mode 1: out_d[0] = sqrt(sum0/sum1) (relative residual).
cudaError_t finalize_partials(const double *partial, int count, int terms, int mode, float *out_f,
                              double *out_d, cudaStream_t s);

// X[k] *= (sum_z P[z*count + k]) / (D[k] + eps)   (nmf_kernels.cu:43-47 with split-K numerator)
cudaError_t euclid_update(float *X, const float *P, int splits, const float *D, long long count,
                          float eps, cudaStream_t s);

// X[k] = max(0, X[k] + (X[k] / D[k]) * (num - D[k])), num = sum_z P[z*count + k]
// (the additive Euclidean update, nmf_kernels.cu:31-38; no epsilon, as there)
cudaError_t additive_update(float *X, const float *P, int splits, const float *D, long long count,
                            cudaStream_t s);

// out[k] = sum_z P[z*count + k] (fixed order)
cudaError_t sum_partials(float *out, const float *P, int splits, long long count, cudaStream_t s);

// KL epilogue: X[k] *= (sum_z P[z*count+k]) / sums[(k / div) % mod]   (nmf_kernels.cu:289,337)
// additive: X[k] = max(0, X[k] + (X[k] / sums[..]) * acc)   (nmf_kernels_additive_divergence.cu:101-104)
cudaError_t kl_update(float *X, const float *P, int splits, const float *sums, long long count,
                      long long div, long long mod, cudaStream_t s, bool additive = false);

// sums[a] = max(sum_i W(i,a), eps) (KernelSumW, nmf_kernels.cu:63-147)
cudaError_t col_sums(const float *W, int n, int r, float eps, float *sums, cudaStream_t s);
// sums[a] = max(sum_u H(a,u), eps) (KernelSumH, nmf_kernels.cu:149-233)
cudaError_t row_sums(const float *H, int r, int m, float eps, float *sums, cudaStream_t s);

// Reference-shaped fused KL kernels over a stored WH (nmf_kernels.cu:247-341), used by the
// compatibility entry points; one launch each, no split-K.
cudaError_t kl_update_h_ref(float *H, const float *W, const float *V, const float *WH,
                            const float *sumW, int n, int m, int r, float eps, cudaStream_t s);
cudaError_t kl_update_w_ref(float *W, const float *H, const float *V, const float *WH,
                            const float *sumH, int n, int m, int r, float eps, cudaStream_t s);
// The same for the additive KL rule (nmf_kernels_additive_divergence.cu:39-185).
cudaError_t akl_update_h_ref(float *H, const float *W, const float *V, const float *WH,
                             const float *sumW, int n, int m, int r, float eps, cudaStream_t s);
cudaError_t akl_update_w_ref(float *W, const float *H, const float *V, const float *WH,
                             const float *sumH, int n, int m, int r, float eps, cudaStream_t s);

}  // namespace gpunmf
