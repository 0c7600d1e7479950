// C entry points around the reference's own CPU NMF (HostNMF), for the tests.
//
// TEST INFRASTRUCTURE ONLY.  This file is compiled by oracle/build.py, in the
// container that holds the reference tree, together with the reference's
// headers src/examples/FacesNMF/HostNMF.h and src/memory/HostMatrix.h taken
// unmodified from where they lie.  The one generated file is a copy of
// src/examples/FacesNMF/Matrix.h whose three member references that g++'s
// two-phase lookup rejects (Matrix.h:64,69-70,79) are qualified with
// this->; it is written into the git-ignored oracle/_ref/ and included first,
// so its include guard (Matrix_h) keeps HostNMF.h from pulling the original.
//
// The library that results (oracle/_ref/libhostnmf_ref.so) is never part of
// the product; it generates the golden vectors under tests/golden/ and pins
// the float transcription in oracle/nmf_oracle.c bit for bit.
#include <cmath>
#include <cstring>
#include "definitions.h"   // reference src/cuda/definitions.h: cudafloat = float
#include "Matrix.h"        // generated, see above
#include "HostNMF.h"       // reference src/examples/FacesNMF/HostNMF.h

static double rel_residual(int n, int m, int r, const float *V, const float *W, const float *H) {
    double num = 0.0, den = 0.0;
    for (int u = 0; u < m; u++)
        for (int i = 0; i < n; i++) {
            double wh = 0.0;
            for (int k = 0; k < r; k++) wh += (double)W[(size_t)k * n + i] * (double)H[(size_t)u * r + k];
            double v = V[(size_t)u * n + i], d = v - wh;
            num += d * d;
            den += v * v;
        }
    return den > 0.0 ? std::sqrt(num / den) : 0.0;
}

// method: 0 multiplicative Euclidean, 1 multiplicative divergence,
// 2 additive Euclidean, 3 additive divergence (HostNMF.h:32-37).  V (n x m), W (n x r), H (r x m) column-major.  W and H
// are inputs and outputs.  resid (nullable) receives the relative Frobenius
// residual after every iteration.
extern "C" int ref_hostnmf_run(int method, int n, int m, int r, const float *V, float *W, float *H,
                               int iters, int updateW, double *resid) {
    if (method < 0 || method > 3) return -1;
    static const NMF_METHOD methods[4] = {MULTIPLICATIVE_EUCLIDEAN, MULTIPLICATIVE_DIVERGENCE, ADDITIVE_EUCLIDEAN,
                                          ADDITIVE_DIVERGENCE};
    HostNMF h(n, m, r);
    std::memcpy(h.V.Pointer(), V, sizeof(float) * (size_t)n * m);
    std::memcpy(h.W.Pointer(), W, sizeof(float) * (size_t)n * r);
    std::memcpy(h.H.Pointer(), H, sizeof(float) * (size_t)r * m);
    for (int it = 0; it < iters; it++) {
        h.DoIteration(methods[method], updateW != 0);
        if (resid) resid[it] = rel_residual(n, m, r, V, h.W.Pointer(), h.H.Pointer());
    }
    std::memcpy(W, h.W.Pointer(), sizeof(float) * (size_t)n * r);
    std::memcpy(H, h.H.Pointer(), sizeof(float) * (size_t)r * m);
    return 0;
}

// Time `iters` iterations of the reference CPU NMF; returns seconds, or -1.
#include <chrono>
extern "C" double ref_hostnmf_time(int method, int n, int m, int r, const float *V, float *W, float *H,
                                   int iters) {
    if (method != 0 && method != 1) return -1.0;
    HostNMF h(n, m, r);
    std::memcpy(h.V.Pointer(), V, sizeof(float) * (size_t)n * m);
    std::memcpy(h.W.Pointer(), W, sizeof(float) * (size_t)n * r);
    std::memcpy(h.H.Pointer(), H, sizeof(float) * (size_t)r * m);
    auto t0 = std::chrono::steady_clock::now();
    for (int it = 0; it < iters; it++)
        h.DoIteration(method == 0 ? MULTIPLICATIVE_EUCLIDEAN : MULTIPLICATIVE_DIVERGENCE, true);
    auto t1 = std::chrono::steady_clock::now();
    std::memcpy(W, h.W.Pointer(), sizeof(float) * (size_t)n * r);
    std::memcpy(H, h.H.Pointer(), sizeof(float) * (size_t)r * m);
    return std::chrono::duration<double>(t1 - t0).count();
}
