/*
 * gpumlib_nmf.hpp — header-only C++ drop-in for GPUMLib's NMF classes.
 *
 * Same namespace, class names, constructors and methods as the reference:
 *   GPUMLib::NMF                                  src/algorithms/nmf/nmf_base.h:45-151
 *   GPUMLib::NMF_MultiplicativeEuclidianDistance  src/algorithms/nmf/nmf_multiplicative_euclidian.h:35-73
 *   GPUMLib::NMF_MultiplicativeDivergence         src/algorithms/nmf/nmf_multiplicative_divergence.h:35-63
 *   GPUMLib::NMF_AdditiveEuclidian                src/algorithms/nmf/nmf_additive_euclidian.h:35-67
 *   GPUMLib::NMF_AdditiveDivergence               src/algorithms/nmf/nmf_additive_divergence.h:35-60
 *   GPUMLib::HostMatrix<T> (the subset the NMF callers use)   src/memory/HostMatrix.h:37-132
 * implemented over the C ABI in gpunmf.h (link with -lgpunmf).
 *
 * Behaviour kept from the reference: inputs must be column-major (asserted,
 * nmf_base.h:92,109-114); H is updated before W; DoIteration(false) skips
 * the W update; QualityImprovement() is the lagged change of the log10
 * quality, 1.0 until three samples exist; GetWH() computes W*H on demand.
 * Differences: CUDA failures throw GPUMLib::NMFError (the reference drops
 * them, nmf_multiplicative_euclidian.cpp:45,66); the random constructor
 * draws W and H from a seeded counter-based generator (the reference uses
 * an unseeded rand(), nmf_base.h:56-61).
 * Additions: Residual() (FP64 relative Frobenius residual on the GPU), ObjectiveKL(),
 * Iterate(k), SetQualityInterval(k) (k > 0: every k-th iteration, 1 by default;
 * 0: never; GPUNMF_QUALITY_WHEN_READY: the reference's rule, a sample whenever the
 * previous read-back is complete), and optional eps / precision arguments on every
 * constructor.
 */
#ifndef GPUMLIB_GB300_NMF_HPP
#define GPUMLIB_GB300_NMF_HPP

#include <cassert>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "gpunmf.h"

namespace GPUMLib {

typedef float cudafloat;

typedef enum { RowMajor, ColumnMajor } StoringOrder;  // src/memory/BaseMatrix.h:33-36

class NMFError : public std::runtime_error {
  public:
    NMFError(gpunmf_status s, const std::string &what) : std::runtime_error(what), status(s) {}
    gpunmf_status status;
};

inline void nmf_check(gpunmf_status s) {
    if (s != GPUNMF_OK) throw NMFError(s, std::string("gpunmf: ") + gpunmf_last_error());
}

//! Host matrix with the storage-order semantics of the reference's HostMatrix.
template <class Type> class HostMatrix {
  public:
    HostMatrix(StoringOrder order = RowMajor) : rows_(0), cols_(0), order_(order) {}
    HostMatrix(size_t rows, size_t columns, StoringOrder order = RowMajor)
        : rows_(rows), cols_(columns), order_(order), data_(rows * columns) {}

    size_t Rows() const { return rows_; }
    size_t Columns() const { return cols_; }
    size_t Elements() const { return rows_ * cols_; }
    bool IsRowMajor() const { return order_ == RowMajor; }
    Type *Pointer() { return data_.empty() ? nullptr : data_.data(); }
    const Type *Pointer() const { return data_.empty() ? nullptr : data_.data(); }

    void ResizeWithoutPreservingData(size_t rows, size_t columns) {
        rows_ = rows;
        cols_ = columns;
        data_.assign(rows * columns, Type());
    }

    //! Zero-copy transpose: flip the storage order and swap the dimensions (BaseMatrix.h:139-145).
    void ReplaceByTranspose() {
        std::swap(rows_, cols_);
        order_ = IsRowMajor() ? ColumnMajor : RowMajor;
    }

    HostMatrix<Type> Transpose() const {
        HostMatrix<Type> t(*this);
        t.ReplaceByTranspose();
        return t;
    }

    Type &operator()(size_t row, size_t column) { return data_[Index(row, column)]; }
    Type operator()(size_t row, size_t column) const { return data_[Index(row, column)]; }

  private:
    size_t Index(size_t row, size_t column) const {
        assert(row < rows_ && column < cols_);
        return IsRowMajor() ? row * cols_ + column : column * rows_ + row;
    }
    size_t rows_, cols_;
    StoringOrder order_;
    std::vector<Type> data_;
};

//! Base class of the NMF algorithms (nmf_base.h:45).
class NMF {
  public:
    NMF(const NMF &) = delete;
    NMF &operator=(const NMF &) = delete;
    virtual ~NMF() {
        if (h_) gpunmf_destroy(h_);
    }

    //! Gets the W matrix (n x r, column-major).
    HostMatrix<cudafloat> GetW() {
        HostMatrix<cudafloat> w(n_, r_, ColumnMajor);
        nmf_check(gpunmf_get_w(h_, w.Pointer()));
        return w;
    }

    //! Gets the H matrix (r x m, column-major).
    HostMatrix<cudafloat> GetH() {
        HostMatrix<cudafloat> h(r_, m_, ColumnMajor);
        nmf_check(gpunmf_get_h(h_, h.Pointer()));
        return h;
    }

    //! Gets the approximation W*H of V (n x m, column-major).
    HostMatrix<cudafloat> GetWH() {
        HostMatrix<cudafloat> wh(n_, m_, ColumnMajor);
        nmf_check(gpunmf_get_wh(h_, wh.Pointer()));
        return wh;
    }

    //! Do an algorithm iteration: adjusts H and (if updateW) W.
    virtual void DoIteration(bool updateW = true) = 0;

    //! Quality improvement caused by the last iterations (lagged; 1.0 initially).
    cudafloat QualityImprovement() const {
        float q = 1.0f;
        nmf_check(gpunmf_quality_improvement(h_, &q));
        return q;
    }

    // ---- additions ----
    void Iterate(int iterations, bool updateW = true) { nmf_check(gpunmf_iterate(h_, iterations, updateW ? 1 : 0)); }
    void SetQualityInterval(int k) { nmf_check(gpunmf_set_quality_interval(h_, k)); }
    double Residual() {
        double r = 0.0;
        nmf_check(gpunmf_residual_fp64(h_, &r));
        return r;
    }
    //! Generalised KL objective sum V log(V / WH) - V + WH, FP64 on the GPU (any rule).
    double ObjectiveKL() {
        double o = 0.0;
        nmf_check(gpunmf_objective_kl_fp64(h_, &o));
        return o;
    }
    gpunmf_handle Handle() const { return h_; }

  protected:
    NMF(int rule, HostMatrix<cudafloat> &v, int r, float eps, int precision, unsigned long long seed)
        : n_((int)v.Rows()), m_((int)v.Columns()), r_(r) {
        assert(!v.IsRowMajor());
        nmf_check(gpunmf_create_random(rule, n_, m_, r_, v.Pointer(), seed, eps, precision, nullptr, &h_));
    }
    NMF(int rule, HostMatrix<cudafloat> &v, HostMatrix<cudafloat> &w, HostMatrix<cudafloat> &h, float eps,
        int precision)
        : n_((int)v.Rows()), m_((int)v.Columns()), r_((int)w.Columns()) {
        assert(!v.IsRowMajor());
        assert(!w.IsRowMajor());
        assert(!h.IsRowMajor());
        assert(v.Rows() == w.Rows() && v.Columns() == h.Columns());
        assert(w.Columns() == h.Rows());
        nmf_check(gpunmf_create(rule, n_, m_, r_, v.Pointer(), w.Pointer(), h.Pointer(), eps, precision, nullptr,
                                &h_));
    }

    gpunmf_handle h_ = nullptr;
    int n_, m_, r_;
};

//! Multiplicative update rules, Euclidean distance (nmf_multiplicative_euclidian.h:35).
class NMF_MultiplicativeEuclidianDistance : public NMF {
  public:
    NMF_MultiplicativeEuclidianDistance(HostMatrix<cudafloat> &v, int r, float eps = GPUNMF_REFERENCE_EPS,
                                        int precision = GPUNMF_FP32, unsigned long long seed = 0)
        : NMF(GPUNMF_EUCLIDEAN, v, r, eps, precision, seed) {}
    NMF_MultiplicativeEuclidianDistance(HostMatrix<cudafloat> &v, HostMatrix<cudafloat> &w,
                                        HostMatrix<cudafloat> &h, float eps = GPUNMF_REFERENCE_EPS,
                                        int precision = GPUNMF_FP32)
        : NMF(GPUNMF_EUCLIDEAN, v, w, h, eps, precision) {}
    void DoIteration(bool updateW = true) override { nmf_check(gpunmf_iterate(h_, 1, updateW ? 1 : 0)); }
};

//! Multiplicative update rules, Kullback-Leibler divergence (nmf_multiplicative_divergence.h:35).
class NMF_MultiplicativeDivergence : public NMF {
  public:
    NMF_MultiplicativeDivergence(HostMatrix<cudafloat> &v, int r, float eps = GPUNMF_REFERENCE_EPS,
                                 int precision = GPUNMF_FP32, unsigned long long seed = 0)
        : NMF(GPUNMF_DIVERGENCE, v, r, eps, precision, seed) {}
    NMF_MultiplicativeDivergence(HostMatrix<cudafloat> &v, HostMatrix<cudafloat> &w, HostMatrix<cudafloat> &h,
                                 float eps = GPUNMF_REFERENCE_EPS, int precision = GPUNMF_FP32)
        : NMF(GPUNMF_DIVERGENCE, v, w, h, eps, precision) {}
    void DoIteration(bool updateW = true) override { nmf_check(gpunmf_iterate(h_, 1, updateW ? 1 : 0)); }
};

//! Additive update rules, Euclidean distance (nmf_additive_euclidian.h:35).  By default it runs
//! what the reference's GPU class runs: that class's H step (nmf_additive_euclidian.cpp:37-42)
//! overwrites a workspace instead of H, so H keeps its initial value and only W is updated.
//! updateH = true applies the additive step to H as well (HostNMF.h:152-190).
class NMF_AdditiveEuclidian : public NMF {
  public:
    NMF_AdditiveEuclidian(HostMatrix<cudafloat> &v, int r, bool updateH = false, int precision = GPUNMF_FP32,
                          unsigned long long seed = 0)
        : NMF(updateH ? GPUNMF_ADDITIVE_EUCLIDEAN : GPUNMF_ADDITIVE_EUCLIDEAN_FIXED_H, v, r,
              GPUNMF_REFERENCE_EPS, precision, seed) {}
    NMF_AdditiveEuclidian(HostMatrix<cudafloat> &v, HostMatrix<cudafloat> &w, HostMatrix<cudafloat> &h,
                          bool updateH = false, int precision = GPUNMF_FP32)
        : NMF(updateH ? GPUNMF_ADDITIVE_EUCLIDEAN : GPUNMF_ADDITIVE_EUCLIDEAN_FIXED_H, v, w, h,
              GPUNMF_REFERENCE_EPS, precision) {}
    void DoIteration(bool updateW = true) override { nmf_check(gpunmf_iterate(h_, 1, updateW ? 1 : 0)); }
};

//! Additive update rules, Kullback-Leibler divergence (nmf_additive_divergence.h:35).
class NMF_AdditiveDivergence : public NMF {
  public:
    NMF_AdditiveDivergence(HostMatrix<cudafloat> &v, int r, float eps = GPUNMF_REFERENCE_EPS,
                           int precision = GPUNMF_FP32, unsigned long long seed = 0)
        : NMF(GPUNMF_ADDITIVE_DIVERGENCE, v, r, eps, precision, seed) {}
    NMF_AdditiveDivergence(HostMatrix<cudafloat> &v, HostMatrix<cudafloat> &w, HostMatrix<cudafloat> &h,
                           float eps = GPUNMF_REFERENCE_EPS, int precision = GPUNMF_FP32)
        : NMF(GPUNMF_ADDITIVE_DIVERGENCE, v, w, h, eps, precision) {}
    void DoIteration(bool updateW = true) override { nmf_check(gpunmf_iterate(h_, 1, updateW ? 1 : 0)); }
};

//! KernelSumW / KernelSumH / KernelNMFquality with the reference's C++ signatures
//! (src/cuda/nmf/nmf_kernels.h:44,64,73); launched on the default stream.
inline void KernelSumW(int blockSize, cudafloat *W, int n, int r, cudafloat *sumW) {
    gpumlib_nmf_sum_w(blockSize, W, n, r, sumW);
}
inline void KernelSumH(int blockSize, cudafloat *H, int r, int m, cudafloat *sumH) {
    gpumlib_nmf_sum_h(blockSize, H, r, m, sumH);
}
inline void KernelNMFquality(int blockSize, cudafloat *V, cudafloat *WH, int n, cudafloat *quality) {
    gpumlib_nmf_quality(blockSize, V, WH, n, quality);
}

}  // namespace GPUMLib

#endif  // GPUMLIB_GB300_NMF_HPP
