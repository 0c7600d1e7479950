/*
 * CPU oracle for GPUMLib's multiplicative-update NMF.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the gpumlib_gb300 product links,
 * loads or calls this file; only the tests, the smoke check and the CPU
 * baseline leg of bench.py do, and only as the checker.
 *
 * Two families of functions:
 *
 *  orc_hostnmf_*  float transcriptions of the reference's CPU NMF, all four
 *                 rules (src/examples/FacesNMF/HostNMF.h:64-233) with the exact
 *                 operation order of its naive products
 *                 (src/examples/FacesNMF/Matrix.h:48-72): every dot product is
 *                 a sequential float accumulation from index 0.  Built with
 *                 -ffp-contract=off so no multiply-add is fused; the result is
 *                 then bit-identical to the reference's own HostNMF compiled
 *                 from its sources (checked against golden vectors made that
 *                 way).  Work is split over threads by output element only, so
 *                 the thread count never changes a result bit.
 *
 *  orc_f64_*      double-precision statements of the GPU classes' rules
 *                 (src/algorithms/nmf/nmf_multiplicative_euclidian.cpp:29-67,
 *                 src/algorithms/nmf/nmf_multiplicative_divergence.cpp:29-50,
 *                 src/cuda/nmf/nmf_kernels.cu:43-47,63-233,247-341), used as
 *                 the accuracy reference for the mixed-precision path.
 *
 * All matrices are column-major: V n x m, W n x r, H r x m.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define IDX(row, col, ld) ((size_t)(col) * (size_t)(ld) + (size_t)(row))

/* ------------------------------------------------------------------ */
/* tiny fork/join helper: run fn(lo, hi, arg) over [0, count) split in */
/* contiguous chunks over nthreads threads                             */
/* ------------------------------------------------------------------ */
typedef void (*range_fn)(long lo, long hi, void *arg);
struct range_job { range_fn fn; long lo, hi; void *arg; };

static void *range_thread(void *p) {
    struct range_job *j = (struct range_job *)p;
    j->fn(j->lo, j->hi, j->arg);
    return NULL;
}

static void parallel_range(long count, int nthreads, range_fn fn, void *arg) {
    if (nthreads <= 1 || count < 2) { fn(0, count, arg); return; }
    if (nthreads > 256) nthreads = 256;
    if (nthreads > count) nthreads = (int)count;
    pthread_t th[256];
    struct range_job jobs[256];
    long chunk = (count + nthreads - 1) / nthreads;
    int started = 0;
    for (int t = 0; t < nthreads; t++) {
        long lo = t * chunk, hi = lo + chunk;
        if (lo >= count) break;
        if (hi > count) hi = count;
        jobs[t].fn = fn; jobs[t].lo = lo; jobs[t].hi = hi; jobs[t].arg = arg;
        if (t == 0) continue;
        if (pthread_create(&th[t], NULL, range_thread, &jobs[t]) != 0) {
            fn(lo, hi, arg);           /* run inline if a thread cannot start */
            jobs[t].fn = NULL;
        }
        started = t + 1;
    }
    fn(jobs[0].lo, jobs[0].hi, arg);
    for (int t = 1; t < started; t++)
        if (jobs[t].fn) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------ */
/* float products in Matrix::Multiply order (Matrix.h:48-57)           */
/* C(row, col) = sum_{l=0}^{K-1} A(row, l) * B(l, col), float, l asc.  */
/* Operands are described by (pointer, ld, transposed) so the views    */
/* the reference makes with ReplaceByTranspose (BaseMatrix.h:139-145)  */
/* are reproduced without copies.                                      */
/* ------------------------------------------------------------------ */
struct fview { const float *p; long ld; int t; };
static inline float fget(struct fview v, long row, long col) {
    return v.t ? v.p[IDX(col, row, v.ld)] : v.p[IDX(row, col, v.ld)];
}

struct fmul_arg { struct fview A, B; float *C; long M, N, K; };

static void fmul_cols(long lo, long hi, void *p) {
    struct fmul_arg *a = (struct fmul_arg *)p;
    for (long c = lo; c < hi; c++)
        for (long r = 0; r < a->M; r++) {
            float value = 0.0f;
            for (long l = 0; l < a->K; l++) value += fget(a->A, r, l) * fget(a->B, l, c);
            a->C[IDX(r, c, a->M)] = value;
        }
}

static void fmul(struct fview A, struct fview B, float *C, long M, long N, long K, int nt) {
    struct fmul_arg a = {A, B, C, M, N, K};
    parallel_range(N, nt, fmul_cols, &a);
}

/* ------------------------------------------------------------------ */
/* HostNMF::DoIteration_ME (HostNMF.h:64-114)                          */
/* ------------------------------------------------------------------ */
struct fupd_arg { float *X; const float *num, *den; float eps; };
static void fupd(long lo, long hi, void *p) {
    struct fupd_arg *a = (struct fupd_arg *)p;
    for (long k = lo; k < hi; k++) a->X[k] *= a->num[k] / (a->den[k] + a->eps);
}

/* ws must hold 2*r*m + r*r + 2*n*r floats */
void orc_hostnmf_me_iter(int n, int m, int r, const float *V, float *W, float *H,
                         int updateW, float eps, float *ws, int nthreads) {
    float *WtV = ws, *WtWH = WtV + (size_t)r * m, *WtW = WtWH + (size_t)r * m;
    float *VHt = WtW + (size_t)r * r, *WHHt = VHt + (size_t)n * r;
    struct fview Wt = {W, n, 1}, Vv = {V, n, 0}, Hv = {H, r, 0}, Ht = {H, r, 1};
    struct fview Wv = {W, n, 0};
    /* WtV = Wt * V ; WtW = Wt * Wt' ; WtWH = WtW * H */
    fmul(Wt, Vv, WtV, r, m, n, nthreads);
    fmul(Wt, Wv, WtW, r, r, n, nthreads);           /* MultiplyBySelfTranspose */
    struct fview WtWv = {WtW, r, 0};
    fmul(WtWv, Hv, WtWH, r, m, r, nthreads);
    struct fupd_arg uh = {H, WtV, WtWH, eps};
    parallel_range((long)r * m, nthreads, fupd, &uh);
    if (!updateW) return;
    /* VHt = V * Ht ; HHt = H * H' ; WHHt = W * HHt */
    fmul(Vv, Ht, VHt, n, r, m, nthreads);
    float *HHt = WtW;
    fmul(Hv, Ht, HHt, r, r, m, nthreads);
    struct fview HHtv = {HHt, r, 0};
    fmul(Wv, HHtv, WHHt, n, r, r, nthreads);
    struct fupd_arg uw = {W, VHt, WHHt, eps};
    parallel_range((long)n * r, nthreads, fupd, &uw);
}

/* ------------------------------------------------------------------ */
/* HostNMF::DoIteration_MD (HostNMF.h:116-150)                         */
/* clamp_sums=1 applies the GPU kernels' guard max(sum, eps)           */
/* (nmf_kernels.cu:104,190), which the CPU code lacks.                 */
/* ------------------------------------------------------------------ */
struct md_arg { int n, m, r; const float *V, *WH; float *W, *H; float eps; int clamp; };

static void md_h(long lo, long hi, void *p) {
    struct md_arg *a = (struct md_arg *)p;
    for (long e = lo; e < hi; e++) {
        long ai = e / a->m, u = e % a->m;      /* HostNMF loops a outer, u inner */
        float sum = 0.0f, sumW = 0.0f;
        for (long i = 0; i < a->n; i++) {
            float w = a->W[IDX(i, ai, a->n)];
            sum += w * a->V[IDX(i, u, a->n)] / (a->WH[IDX(i, u, a->n)] + a->eps);
            sumW += w;
        }
        if (a->clamp && sumW < a->eps) sumW = a->eps;
        a->H[IDX(ai, u, a->r)] *= sum / sumW;
    }
}

static void md_w(long lo, long hi, void *p) {
    struct md_arg *a = (struct md_arg *)p;
    for (long e = lo; e < hi; e++) {
        long i = e / a->r, ai = e % a->r;
        float sum = 0.0f, sumH = 0.0f;
        for (long u = 0; u < a->m; u++) {
            float h = a->H[IDX(ai, u, a->r)];
            sum += h * a->V[IDX(i, u, a->n)] / (a->WH[IDX(i, u, a->n)] + a->eps);
            sumH += h;
        }
        if (a->clamp && sumH < a->eps) sumH = a->eps;
        a->W[IDX(i, ai, a->n)] *= sum / sumH;
    }
}

/* ws must hold n*m floats (WH) */
void orc_hostnmf_md_iter(int n, int m, int r, const float *V, float *W, float *H,
                         int updateW, float eps, int clamp_sums, float *ws, int nthreads) {
    struct fview Wv = {W, n, 0}, Hv = {H, r, 0};
    float *WH = ws;
    fmul(Wv, Hv, WH, n, m, r, nthreads);
    struct md_arg a = {n, m, r, V, WH, W, H, eps, clamp_sums};
    parallel_range((long)r * m, nthreads, md_h, &a);
    if (!updateW) return;
    fmul(Wv, Hv, WH, n, m, r, nthreads);
    parallel_range((long)n * r, nthreads, md_w, &a);
}

/* ------------------------------------------------------------------ */
/* HostNMF::DoIteration_AE (HostNMF.h:152-190): additive Euclidean     */
/* ------------------------------------------------------------------ */
struct fadd_arg { float *X; const float *d1, *d2; };
static void fadd(long lo, long hi, void *p) {
    struct fadd_arg *a = (struct fadd_arg *)p;
    for (long k = lo; k < hi; k++) {
        float x = a->X[k];
        float d2 = a->d2[k];
        float lr = x / d2;
        x += lr * (a->d1[k] - d2);
        a->X[k] = (x < 0.0f) ? 0.0f : x;
    }
}

/* ws must hold 2*r*m + r*r + 2*n*r floats.  skip_h = 1 reproduces the GPU class
 * NMF_AdditiveEuclidian (nmf_additive_euclidian.cpp:42), whose H step writes into a
 * workspace instead of H, so H never changes. */
void orc_hostnmf_ae_iter(int n, int m, int r, const float *V, float *W, float *H,
                         int updateW, int skip_h, float *ws, int nthreads) {
    float *WtV = ws, *WtWH = WtV + (size_t)r * m, *WtW = WtWH + (size_t)r * m;
    float *VHt = WtW + (size_t)r * r, *WHHt = VHt + (size_t)n * r;
    struct fview Wt = {W, n, 1}, Vv = {V, n, 0}, Hv = {H, r, 0}, Ht = {H, r, 1};
    struct fview Wv = {W, n, 0};
    if (!skip_h) {
        fmul(Wt, Vv, WtV, r, m, n, nthreads);
        fmul(Wt, Wv, WtW, r, r, n, nthreads);
        struct fview WtWv = {WtW, r, 0};
        fmul(WtWv, Hv, WtWH, r, m, r, nthreads);
        struct fadd_arg uh = {H, WtV, WtWH};
        parallel_range((long)r * m, nthreads, fadd, &uh);
    }
    if (!updateW) return;
    fmul(Vv, Ht, VHt, n, r, m, nthreads);
    float *HHt = WtW;
    fmul(Hv, Ht, HHt, r, r, m, nthreads);
    struct fview HHtv = {HHt, r, 0};
    fmul(Wv, HHtv, WHHt, n, r, r, nthreads);
    struct fadd_arg uw = {W, VHt, WHHt};
    parallel_range((long)n * r, nthreads, fadd, &uw);
}

/* ------------------------------------------------------------------ */
/* HostNMF::DoIteration_AD (HostNMF.h:192-233): additive KL            */
/* clamp_sums=1 applies the GPU kernels' max(sum, eps) on the sums.    */
/* ------------------------------------------------------------------ */
static void ad_h(long lo, long hi, void *p) {
    struct md_arg *a = (struct md_arg *)p;
    for (long e = lo; e < hi; e++) {
        long ai = e / a->m, u = e % a->m;
        float sum = 0.0f, sumW = 0.0f;
        for (long i = 0; i < a->n; i++) {
            float w = a->W[IDX(i, ai, a->n)];
            sum += w * a->V[IDX(i, u, a->n)] / (a->WH[IDX(i, u, a->n)] + a->eps) - w;
            sumW += w;
        }
        if (a->clamp && sumW < a->eps) sumW = a->eps;
        float h = a->H[IDX(ai, u, a->r)];
        float lr = h / sumW;
        h += lr * sum;
        a->H[IDX(ai, u, a->r)] = (h < 0.0f) ? 0.0f : h;
    }
}

static void ad_w(long lo, long hi, void *p) {
    struct md_arg *a = (struct md_arg *)p;
    for (long e = lo; e < hi; e++) {
        long i = e / a->r, ai = e % a->r;
        float sum = 0.0f, sumH = 0.0f;
        for (long u = 0; u < a->m; u++) {
            float h = a->H[IDX(ai, u, a->r)];
            sum += h * a->V[IDX(i, u, a->n)] / (a->WH[IDX(i, u, a->n)] + a->eps) - h;
            sumH += h;
        }
        if (a->clamp && sumH < a->eps) sumH = a->eps;
        float w = a->W[IDX(i, ai, a->n)];
        float lr = w / sumH;
        w += lr * sum;
        a->W[IDX(i, ai, a->n)] = (w < 0.0f) ? 0.0f : w;
    }
}

/* ws must hold n*m floats (WH) */
void orc_hostnmf_ad_iter(int n, int m, int r, const float *V, float *W, float *H,
                         int updateW, float eps, int clamp_sums, float *ws, int nthreads) {
    struct fview Wv = {W, n, 0}, Hv = {H, r, 0};
    float *WH = ws;
    fmul(Wv, Hv, WH, n, m, r, nthreads);
    struct md_arg a = {n, m, r, V, WH, W, H, eps, clamp_sums};
    parallel_range((long)r * m, nthreads, ad_h, &a);
    if (!updateW) return;
    fmul(Wv, Hv, WH, n, m, r, nthreads);
    parallel_range((long)n * r, nthreads, ad_w, &a);
}

/* W*H in Matrix::Multiply order (the WH that GetWH returns on the CPU) */
void orc_hostnmf_wh(int n, int m, int r, const float *W, const float *H, float *WH, int nthreads) {
    struct fview Wv = {W, n, 0}, Hv = {H, r, 0};
    fmul(Wv, Hv, WH, n, m, r, nthreads);
}

/* ------------------------------------------------------------------ */
/* double-precision statements of the GPU rules                        */
/* ------------------------------------------------------------------ */
struct dmul_arg { const double *A; long lda; int ta; const double *B; long ldb; int tb;
                  double *C; long M, N, K; };
static void dmul_cols(long lo, long hi, void *p) {
    struct dmul_arg *a = (struct dmul_arg *)p;
    for (long c = lo; c < hi; c++)
        for (long r = 0; r < a->M; r++) {
            double s = 0.0;
            for (long l = 0; l < a->K; l++) {
                double x = a->ta ? a->A[IDX(l, r, a->lda)] : a->A[IDX(r, l, a->lda)];
                double y = a->tb ? a->B[IDX(c, l, a->ldb)] : a->B[IDX(l, c, a->ldb)];
                s += x * y;
            }
            a->C[IDX(r, c, a->M)] = s;
        }
}
static void dmul(const double *A, long lda, int ta, const double *B, long ldb, int tb,
                 double *C, long M, long N, long K, int nt) {
    struct dmul_arg a = {A, lda, ta, B, ldb, tb, C, M, N, K};
    parallel_range(N, nt, dmul_cols, &a);
}

/* Euclidean rule (nmf_multiplicative_euclidian.cpp:29-67, kernel nmf_kernels.cu:43-47).
 * ws: 2*r*m + r*r + 2*n*r doubles. */
void orc_f64_me_iter(int n, int m, int r, const double *V, double *W, double *H,
                     int updateW, double eps, double *ws, int nthreads) {
    double *WtV = ws, *WtWH = WtV + (size_t)r * m, *G = WtWH + (size_t)r * m;
    double *VHt = G + (size_t)r * r, *WHHt = VHt + (size_t)n * r;
    dmul(W, n, 1, V, n, 0, WtV, r, m, n, nthreads);
    dmul(W, n, 1, W, n, 0, G, r, r, n, nthreads);
    dmul(G, r, 0, H, r, 0, WtWH, r, m, r, nthreads);
    for (size_t k = 0; k < (size_t)r * m; k++) H[k] *= WtV[k] / (WtWH[k] + eps);
    if (!updateW) return;
    dmul(V, n, 0, H, r, 1, VHt, n, r, m, nthreads);
    dmul(H, r, 0, H, r, 1, G, r, r, m, nthreads);
    dmul(W, n, 0, G, r, 0, WHHt, n, r, r, nthreads);
    for (size_t k = 0; k < (size_t)n * r; k++) W[k] *= VHt[k] / (WHHt[k] + eps);
}

struct dmd_arg { int n, m, r; const double *V, *WH; double *W, *H, *sum; double eps; };
static void dmd_h(long lo, long hi, void *p) {
    struct dmd_arg *a = (struct dmd_arg *)p;
    for (long u = lo; u < hi; u++) {
        double acc[512];
        int r = a->r;
        for (int k = 0; k < r; k++) acc[k] = 0.0;
        for (long i = 0; i < a->n; i++) {
            double q = a->V[IDX(i, u, a->n)] / (a->WH[IDX(i, u, a->n)] + a->eps);
            for (int k = 0; k < r; k++) acc[k] += a->W[IDX(i, k, a->n)] * q;
        }
        for (int k = 0; k < r; k++) a->H[IDX(k, u, r)] *= acc[k] / a->sum[k];
    }
}
static void dmd_w(long lo, long hi, void *p) {
    struct dmd_arg *a = (struct dmd_arg *)p;
    int r = a->r;
    for (long i = lo; i < hi; i++) {
        double acc[512];
        for (int k = 0; k < r; k++) acc[k] = 0.0;
        for (long u = 0; u < a->m; u++) {
            double q = a->V[IDX(i, u, a->n)] / (a->WH[IDX(i, u, a->n)] + a->eps);
            for (int k = 0; k < r; k++) acc[k] += a->H[IDX(k, u, r)] * q;
        }
        for (int k = 0; k < r; k++) a->W[IDX(i, k, a->n)] *= acc[k] / a->sum[k];
    }
}

/* KL rule with the GPU's clamp of the row/column sums
 * (nmf_multiplicative_divergence.cpp:29-50; nmf_kernels.cu:63-233,247-341).
 * ws: n*m + r doubles.  r <= 512. */
int orc_f64_md_iter(int n, int m, int r, const double *V, double *W, double *H,
                    int updateW, double eps, double *ws, int nthreads) {
    if (r > 512) return -1;
    double *WH = ws, *sum = ws + (size_t)n * m;
    dmul(W, n, 0, H, r, 0, WH, n, m, r, nthreads);
    for (int k = 0; k < r; k++) {
        double s = 0.0;
        for (long i = 0; i < n; i++) s += W[IDX(i, k, n)];
        sum[k] = s < eps ? eps : s;
    }
    struct dmd_arg a = {n, m, r, V, WH, W, H, sum, eps};
    parallel_range(m, nthreads, dmd_h, &a);
    if (!updateW) return 0;
    dmul(W, n, 0, H, r, 0, WH, n, m, r, nthreads);
    for (int k = 0; k < r; k++) {
        double s = 0.0;
        for (long u = 0; u < m; u++) s += H[IDX(k, u, r)];
        sum[k] = s < eps ? eps : s;
    }
    parallel_range(n, nthreads, dmd_w, &a);
    return 0;
}

/* ------------------------------------------------------------------ */
/* reductions                                                          */
/* ------------------------------------------------------------------ */

/* The reference's quality value (nmf_kernels_quality.cu:29-41):
 * sum_k V[k]*log10(WH[k] + eps) - WH[k], evaluated per element in float
 * as the kernel does, accumulated in double here. */
double orc_quality(long count, const float *V, const float *WH, float eps) {
    double s = 0.0;
    for (long k = 0; k < count; k++) {
        float wh = WH[k];
        float t = V[k] * log10f(wh + eps) - wh;
        s += (double)t;
    }
    return s;
}

/* relative Frobenius residual ||V - W H||_F / ||V||_F, all in double,
 * from float inputs */
struct res_arg { int n, m, r; const float *V, *W, *H; double *num, *den; };
static void res_cols(long lo, long hi, void *p) {
    struct res_arg *a = (struct res_arg *)p;
    double num = 0.0, den = 0.0;
    for (long u = lo; u < hi; u++)
        for (long i = 0; i < a->n; i++) {
            double wh = 0.0;
            for (int k = 0; k < a->r; k++)
                wh += (double)a->W[IDX(i, k, a->n)] * (double)a->H[IDX(k, u, a->r)];
            double v = a->V[IDX(i, u, a->n)], d = v - wh;
            num += d * d; den += v * v;
        }
    a->num[lo] = num; a->den[lo] = den;  /* slot lo is unique per chunk */
}
double orc_residual(int n, int m, int r, const float *V, const float *W, const float *H,
                    int nthreads) {
    double *num = (double *)calloc((size_t)m, sizeof(double));
    double *den = (double *)calloc((size_t)m, sizeof(double));
    if (!num || !den) { free(num); free(den); return -1.0; }
    struct res_arg a = {n, m, r, V, W, H, num, den};
    parallel_range(m, nthreads, res_cols, &a);
    double sn = 0.0, sd = 0.0;
    for (long u = 0; u < m; u++) { sn += num[u]; sd += den[u]; }
    free(num); free(den);
    return sd > 0.0 ? sqrt(sn / sd) : 0.0;
}
