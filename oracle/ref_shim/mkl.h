/*
 * Stand-in <mkl.h> used ONLY to compile the reference's HLanc.hpp into the
 * checker library oracle/_ref/libhlanc_ref.so (oracle/build_ref.sh).  Test
 * infrastructure: the product never includes this file.
 *
 * Intel MKL is not installed in the development image.  The reference calls
 * these MKL entry points (HLanc.hpp:452-465, 911-940, 1372-1837); each is
 * mapped to the scipy-bundled LP64 OpenBLAS (exported names carry a
 * "scipy_" prefix; Fortran character arguments take hidden lengths), except:
 *   - mkl_dcsrmv: restated here for alpha=1, beta=0, zero-based, "G"/"S"
 *     (lower) descriptors, the only way the reference calls it;
 *   - dlarnv: its only caller is dgetv0 (HLanc.hpp:1372); when the wrapper
 *     has set hlanc_ref_start_vector the start vector is copied from there,
 *     so the reference and the GPU build start from identical vectors.
 * Two CUDA 13 compatibility shims let the header's GPU classes compile:
 * cusparseDcsrmv (removed from cuSPARSE) is a stub that returns
 * CUSPARSE_STATUS_NOT_SUPPORTED and is never called on the CPU path, and the
 * cudaPointerAttributes field memoryType is spelled `type` today.
 */
#pragma once
#include <cmath>
#include <cstddef>
#include <cstring>
#include <cuda_runtime.h>
#include <cusparse.h>

extern "C" {
double scipy_cblas_dnrm2(int n, const double *x, int incx);
void scipy_cblas_dgemv(int order, int trans, int m, int n, double alpha, const double *a, int lda,
                       const double *x, int incx, double beta, double *y, int incy);
void scipy_dsteqr_(const char *compz, const int *n, double *d, double *e, double *z, const int *ldz,
                   double *work, int *info, size_t);
void scipy_dlartg_(const double *f, const double *g, double *c, double *s, double *r);
void scipy_dgeqr2_(const int *m, const int *n, double *a, const int *lda, double *tau, double *work,
                   int *info);
void scipy_dorm2r_(const char *side, const char *trans, const int *m, const int *n, const int *k,
                   const double *a, const int *lda, const double *tau, double *c, const int *ldc,
                   double *work, int *info, size_t, size_t);
double scipy_dlamch_(const char *cmach, size_t);
void scipy_dlaset_(const char *uplo, const int *m, const int *n, const double *alpha,
                   const double *beta, double *a, const int *lda, size_t);
void scipy_dlarnv_(const int *idist, int *iseed, const int *n, double *x);
}

extern const double *hlanc_ref_start_vector;

enum CBLAS_LAYOUT { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };

inline double cblas_dnrm2(int n, const double *x, int incx) { return scipy_cblas_dnrm2(n, x, incx); }
inline void cblas_dgemv(CBLAS_LAYOUT o, CBLAS_TRANSPOSE t, int m, int n, double alpha,
                        const double *a, int lda, const double *x, int incx, double beta, double *y,
                        int incy) {
    scipy_cblas_dgemv((int)o, (int)t, m, n, alpha, a, lda, x, incx, beta, y, incy);
}
inline void dsteqr(const char *compz, int *n, double *d, double *e, double *z, int *ldz,
                   double *work, int *info) {
    scipy_dsteqr_(compz, n, d, e, z, ldz, work, info, 1);
}
inline void dlartg(double *f, double *g, double *c, double *s, double *r) { scipy_dlartg_(f, g, c, s, r); }
inline void dgeqr2(int *m, int *n, double *a, int *lda, double *tau, double *work, int *info) {
    scipy_dgeqr2_(m, n, a, lda, tau, work, info);
}
inline void dorm2r(const char *side, const char *trans, int *m, int *n, int *k, double *a, int *lda,
                   double *tau, double *c, int *ldc, double *work, int *info) {
    scipy_dorm2r_(side, trans, m, n, k, a, lda, tau, c, ldc, work, info, 1, 1);
}
inline double dlamch(const char *c) { return scipy_dlamch_(c, 1); }
inline void dlaset(const char *uplo, int *m, int *n, const double *alpha, const double *beta,
                   double *a, int *lda) {
    scipy_dlaset_(uplo, m, n, alpha, beta, a, lda, 1);
}
inline void dlarnv(int *idist, int *iseed, int *n, double *x) {
    if (hlanc_ref_start_vector) std::memcpy(x, hlanc_ref_start_vector, sizeof(double) * (size_t)*n);
    else scipy_dlarnv_(idist, iseed, n, x);
}

/* y = A x for the descriptors the reference passes: "GLNC" (general) or
 * "SLNC" (symmetric, lower triangle used, non-unit diagonal, zero-based). */
inline void mkl_dcsrmv(const char *transa, const int *m, const int *k, const double *alpha,
                       const char *matdescra, const double *val, const int *indx, const int *pntrb,
                       const int *pntre, const double *x, const double *beta, double *y) {
    (void)transa; (void)k;
    const int rows = *m;
    for (int i = 0; i < rows; ++i) y[i] = (*beta == 0.0) ? 0.0 : *beta * y[i];
    if (matdescra[0] == 'S') {
        for (int r = 0; r < rows; ++r)
            for (int i = pntrb[r]; i < pntre[r]; ++i) {
                int c = indx[i];
                if (c > r) continue;
                y[r] += *alpha * val[i] * x[c];
                if (c < r) y[c] += *alpha * val[i] * x[r];
            }
    } else {
        for (int r = 0; r < rows; ++r) {
            double s = 0.0;
            for (int i = pntrb[r]; i < pntre[r]; ++i) s += val[i] * x[indx[i]];
            y[r] += *alpha * s;
        }
    }
}

/* CUDA 13 compatibility */
#define memoryType type
inline cusparseStatus_t cusparseDcsrmv(cusparseHandle_t, cusparseOperation_t, int, int, int,
                                       const double *, const cusparseMatDescr_t, const double *,
                                       const int *, const int *, const double *, const double *,
                                       double *) {
    return CUSPARSE_STATUS_NOT_SUPPORTED;
}
