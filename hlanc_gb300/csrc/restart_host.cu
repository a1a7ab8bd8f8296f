// restart_host.cu -- the O(ncv^2) part of a restart cycle, on the host CPU.
//
// Measured on GB300: a dependent chain of scalar FP64 instructions costs
// about 60 SM cycles per instruction on the device (the FP64 pipe issues a
// warp instruction over many cycles), so the reference's sequential
// tridiagonal QR and Givens bulge chase (ncv <= 128) took ~15 ms per restart
// as a one-thread device kernel.  The same work takes well under a
// millisecond on one Grace core.  The engine already synchronises once per
// restart cycle to read the problem state, so these routines run there,
// between the device's extension of the Lanczos factorisation and its V*Q
// basis update; every O(n) operation stays on the GPU.
//
// Algorithms (written from their textbook definitions):
//  - tridiagonal eigenvalues + last eigenvector row: implicit symmetric QR
//    with Wilkinson shift (Golub & Van Loan 4e, Alg. 8.3.2 / 8.3.3);
//  - Givens rotations with the LAPACK >= 3.10 convention (c >= 0, r signed
//    like f; Anderson, ACM TOMS 2017);
//  - Householder QR and the explicit orthogonal factor (G&VL Alg. 5.1.1).
// Control flow follows the reference's ds_solver (HLanc.hpp:1650-1850).
#include <float.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "restart_host.h"

namespace hlanc {
namespace host {

static void givens(double f, double g, double &c, double &s, double &r) {
    if (g == 0.0) { c = 1.0; s = 0.0; r = f; return; }
    if (f == 0.0) { c = 0.0; s = copysign(1.0, g); r = fabs(g); return; }
    const double f1 = fabs(f), g1 = fabs(g);
    const double rtmin = 1.4916681462400413e-154, rtmax = 9.4807519081091774e+153;
    if (f1 > rtmin && f1 < rtmax && g1 > rtmin && g1 < rtmax) {
        const double d = sqrt(f * f + g * g);
        c = f1 / d;
        r = copysign(d, f);
        s = g / r;
    } else {
        const double u = fmin(DBL_MAX, fmax(DBL_MIN, fmax(f1, g1)));
        const double fs = f / u, gs = g / u;
        const double d = sqrt(fs * fs + gs * gs);
        c = fabs(fs) / d;
        r = copysign(d, f);
        s = gs / r;
        r *= u;
    }
}

// sqrt(a^2 + b^2): the plain formula when neither square can overflow or
// underflow, hypot otherwise (hypot's scaling costs more than the rest of
// a QR rotation; the tridiagonal QR is most of a host restart).
static inline double pyth(double a, double b) {
    const double fa = fabs(a), fb = fabs(b);
    const double big = fa > fb ? fa : fb;
    const double rtmin = 1.4916681462400413e-154, rtmax = 9.4807519081091774e+153;
    if (big < rtmax && (big > rtmin || big == 0.0) && (fa > rtmin || fa == 0.0) && (fb > rtmin || fb == 0.0))
        return sqrt(a * a + b * b);
    return hypot(a, b);
}

// Eigenvalues (ascending) of the symmetric tridiagonal (d[n], e[n-1]);
// zl (optional) is rotated as the last row of the eigenvector matrix, Z
// (optional, n x n, ldz) receives all eigenvectors.  0 on success.
int tridiag_eig(int n, double *d, double *e, double *zl, double *Z, int ldz) {
    const double eps = DBL_EPSILON * 0.5;
    if (Z)
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) Z[i + (size_t)j * ldz] = (i == j) ? 1.0 : 0.0;
    int hi = n - 1;
    long iters = 0;
    while (hi > 0) {
        for (int i = 0; i < hi; ++i)
            if (fabs(e[i]) <= eps * (fabs(d[i]) + fabs(d[i + 1])) || fabs(e[i]) < DBL_MIN) e[i] = 0.0;
        while (hi > 0 && e[hi - 1] == 0.0) --hi;
        if (hi == 0) break;
        int lo = hi - 1;
        while (lo > 0 && e[lo - 1] != 0.0) --lo;
        if (++iters > 30L * n) return 1;
        const double dd = 0.5 * (d[hi - 1] - d[hi]);
        const double b = e[hi - 1];
        const double den = dd + copysign(pyth(dd, b), dd);
        const double mu = (den != 0.0) ? d[hi] - b * (b / den) : d[hi] - fabs(b);
        double x = d[lo] - mu, zz = e[lo];
        for (int k = lo; k < hi; ++k) {
            const double r = pyth(x, zz);
            double c = 1.0, s = 0.0;
            if (r != 0.0) { c = x / r; s = zz / r; }
            if (k > lo) e[k - 1] = r;
            const double ak = d[k], ak1 = d[k + 1], bk = e[k];
            d[k] = c * c * ak + 2.0 * c * s * bk + s * s * ak1;
            d[k + 1] = s * s * ak - 2.0 * c * s * bk + c * c * ak1;
            e[k] = c * s * (ak1 - ak) + (c * c - s * s) * bk;
            if (k < hi - 1) {
                zz = s * e[k + 1];
                e[k + 1] = c * e[k + 1];
                x = e[k];
            }
            if (zl) {
                const double a0 = zl[k], a1 = zl[k + 1];
                zl[k] = c * a0 + s * a1;
                zl[k + 1] = -s * a0 + c * a1;
            }
            if (Z) {
                double *zk = Z + (size_t)k * ldz, *zk1 = Z + (size_t)(k + 1) * ldz;
                for (int i = 0; i < n; ++i) {
                    const double a0 = zk[i], a1 = zk1[i];
                    zk[i] = c * a0 + s * a1;
                    zk1[i] = -s * a0 + c * a1;
                }
            }
        }
    }
    for (int i = 0; i < n - 1; ++i) {          // ascending, selection sort
        int k = i;
        for (int j = i + 1; j < n; ++j)
            if (d[j] < d[k]) k = j;
        if (k != i) {
            const double t = d[i]; d[i] = d[k]; d[k] = t;
            if (zl) { const double tz = zl[i]; zl[i] = zl[k]; zl[k] = tz; }
            if (Z)
                for (int r = 0; r < n; ++r) {
                    const double tz = Z[r + (size_t)i * ldz];
                    Z[r + (size_t)i * ldz] = Z[r + (size_t)k * ldz];
                    Z[r + (size_t)k * ldz] = tz;
                }
        }
    }
    return 0;
}

// Cyclic Jacobi for a dense symmetric matrix (Golub & Van Loan 4e,
// Alg. 8.5.1 "symSchur2" and Alg. 8.5.3): rotations zero each off-diagonal
// pair in turn until the off-diagonal norm is below n eps ||A||_F (the
// rounding level of the rotations themselves).
int sym_eig_jacobi(int n, double *A, double *w, double *Z) {
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) Z[i + (size_t)j * n] = (i == j) ? 1.0 : 0.0;
    double fro = 0.0;
    for (int i = 0; i < n * n; ++i) fro += A[i] * A[i];
    fro = sqrt(fro);
    const double eps = DBL_EPSILON * 0.5;
    int ok = 0;
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = 0.0;
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i)
                if (i != j) off += A[i + (size_t)j * n] * A[i + (size_t)j * n];
        if (sqrt(off) <= n * eps * fro || fro == 0.0) { ok = 1; break; }
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[p + (size_t)q * n];
                if (apq == 0.0) continue;
                const double tau = (A[q + (size_t)q * n] - A[p + (size_t)p * n]) / (2.0 * apq);
                const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                const double c = 1.0 / sqrt(1.0 + t * t), sn = t * c;
                for (int k = 0; k < n; ++k) {           // A <- A J (columns p, q)
                    const double akp = A[k + (size_t)p * n], akq = A[k + (size_t)q * n];
                    A[k + (size_t)p * n] = c * akp - sn * akq;
                    A[k + (size_t)q * n] = sn * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {           // A <- J^T A (rows p, q)
                    const double apk = A[p + (size_t)k * n], aqk = A[q + (size_t)k * n];
                    A[p + (size_t)k * n] = c * apk - sn * aqk;
                    A[q + (size_t)k * n] = sn * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {           // Z <- Z J
                    const double zkp = Z[k + (size_t)p * n], zkq = Z[k + (size_t)q * n];
                    Z[k + (size_t)p * n] = c * zkp - sn * zkq;
                    Z[k + (size_t)q * n] = sn * zkp + c * zkq;
                }
            }
    }
    for (int i = 0; i < n; ++i) w[i] = A[i + (size_t)i * n];
    for (int i = 0; i < n - 1; ++i) {             // ascending, columns of Z alike
        int k = i;
        for (int j = i + 1; j < n; ++j)
            if (w[j] < w[k]) k = j;
        if (k != i) {
            const double t = w[i]; w[i] = w[k]; w[k] = t;
            for (int r = 0; r < n; ++r) {
                const double tz = Z[r + (size_t)i * n];
                Z[r + (size_t)i * n] = Z[r + (size_t)k * n];
                Z[r + (size_t)k * n] = tz;
            }
        }
    }
    return ok ? 0 : 1;
}

// dsgets (HLanc.hpp:1387-1401), stable insertion sorts.
static void dsgets(int nev, int np, double *ritz, double *bounds) {
    const int m = nev + np;
    for (int i = 1; i < m; ++i) {
        const double a = ritz[i], b = bounds[i];
        int j = i - 1;
        while (j >= 0 && a < ritz[j]) { ritz[j + 1] = ritz[j]; bounds[j + 1] = bounds[j]; --j; }
        ritz[j + 1] = a; bounds[j + 1] = b;
    }
    for (int i = 1; i < np; ++i) {
        const double a = ritz[i], b = bounds[i];
        int j = i - 1;
        while (j >= 0 && b > bounds[j]) { ritz[j + 1] = ritz[j]; bounds[j + 1] = bounds[j]; --j; }
        ritz[j + 1] = a; bounds[j + 1] = b;
    }
}

// dsapps (HLanc.hpp:1485-1589): np shifted QR steps on T = (alpha = h[m..],
// beta = h[0..]) through a Givens bulge chase, accumulated in Q (m x m).
static void dsapps_T(int m, int np, const double *shift, double *h, double *Q) {
    const double epsmch = DBL_EPSILON * 0.5;
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) Q[i + (size_t)j * m] = (i == j) ? 1.0 : 0.0;
    int itop = 1;
    double c = 0.0, s = 0.0, r = 0.0;
    auto rotq = [&](int col, int lim) {
        double *q0 = Q + (size_t)(col - 1) * m, *q1 = Q + (size_t)col * m;
        for (int j = 0; j < lim; ++j) {
            const double a = q0[j], b = q1[j];
            q0[j] = c * a + s * b;
            q1[j] = -s * a + c * b;
        }
    };
    for (int jj = 1; jj <= np; ++jj) {
        int istart = itop;
        for (;;) {
            int iend = m;
            for (int i = istart; i <= m - 1; ++i) {
                const double big = fabs(h[m + i - 1]) + fabs(h[m + i]);
                if (h[i] <= epsmch * big) { h[i] = 0.0; iend = i; break; }
            }
            if (istart < iend) {
                double f = h[istart + m - 1] - shift[jj - 1];
                double g = h[istart];
                givens(f, g, c, s, r);
                const double a1 = c * h[istart + m - 1] + s * h[istart];
                const double a2 = c * h[istart] + s * h[istart + m];
                const double a4 = c * h[istart + m] - s * h[istart];
                const double a3 = c * h[istart] - s * h[istart + m - 1];
                h[istart + m - 1] = c * a1 + s * a2;
                h[istart + m] = c * a4 - s * a3;
                h[istart] = c * a3 + s * a4;
                rotq(istart, istart + jj < m ? istart + jj : m);
                for (int i = istart + 1; i <= iend - 1; ++i) {
                    f = h[i - 1];
                    g = s * h[i];
                    h[i] = c * h[i];
                    givens(f, g, c, s, r);
                    if (r < 0.0) { r = -r; c = -c; s = -s; }
                    h[i - 1] = r;
                    const double b1 = c * h[i + m - 1] + s * h[i];
                    const double b2 = c * h[i] + s * h[i + m];
                    const double b3 = c * h[i] - s * h[i + m - 1];
                    const double b4 = c * h[i + m] - s * h[i];
                    h[i + m - 1] = c * b1 + s * b2;
                    h[i + m] = c * b4 - s * b3;
                    h[i] = c * b3 + s * b4;
                    rotq(i, i + jj < m ? i + jj : m);
                }
            }
            istart = iend + 1;
            if (h[iend - 1] < 0.0) {
                h[iend - 1] = -h[iend - 1];
                double *qc = Q + (size_t)(iend - 1) * m;
                for (int i = 0; i < m; ++i) qc[i] = -qc[i];
            }
            if (iend < m) continue;
            for (int i = itop; i <= m - 1; ++i) {
                if (h[i] > 0.0) break;
                ++itop;
            }
            break;
        }
    }
    for (int i = itop; i <= m - 1; ++i) {
        const double big = fabs(h[i + m - 1]) + fabs(h[i + m]);
        if (h[i] <= epsmch * big) h[i] = 0.0;
    }
}

int restart(RestartIO &io) {
    const int m = io.ncv;
    std::vector<double> d(m), e(m), zl(m), ritz(m), bounds(m);
    double *h = io.h;
    for (int i = 0; i < m; ++i) {
        d[i] = h[m + i];
        e[i] = (i + 1 < m) ? h[i + 1] : 0.0;
        zl[i] = (i == m - 1) ? 1.0 : 0.0;
    }
    io.iter += 1;
    if (tridiag_eig(m, d.data(), e.data(), zl.data(), nullptr, 0)) return io.status = RS_FAILED;
    for (int i = 0; i < m; ++i) {
        ritz[i] = d[i];
        bounds[i] = io.rnorm * fabs(zl[i]);              // HLanc.hpp:1693-1695
        io.ritz_s[i] = ritz[i];                          // HLanc.hpp:1697-1698
        io.bnds_s[i] = bounds[i];
    }
    int nev = io.nev0, np = io.np0;
    dsgets(nev, np, ritz.data(), bounds.data());
    int nconv = 0;                                       // dsconv, HLanc.hpp:1377-1384
    for (int i = 0; i < nev; ++i) nconv += bounds[np + i] <= io.tol * fmax(io.eps23, fabs(ritz[np + i]));
    for (int jj = 0; jj < np; ++jj)                      // HLanc.hpp:1708-1713
        if (bounds[jj] == 0.0) { --np; ++nev; }
    io.nconv = nconv;
    if (nconv >= io.nev0 || np == 0) return io.status = (nconv >= io.nev0) ? RS_CONVERGED : RS_NOT_CONVERGED;
    if (io.iter >= io.max_iter) return io.status = RS_NOT_CONVERGED;
    const int nevbef = nev;                              // HLanc.hpp:1719-1730
    nev += (nconv < np / 2) ? nconv : np / 2;
    if (nev == 1 && m >= 6) nev = m / 2;
    else if (nev == 1 && m > 2) nev = 2;
    np = m - nev;
    if (nevbef < nev) dsgets(nev, np, ritz.data(), bounds.data());
    dsapps_T(m, np, ritz.data(), h, io.Q);
    io.nev = nev;
    io.np = np;
    return io.status = RS_APPLY;
}

int finalize(FinalizeIO &io) {
    const int m = io.ncv, nev0 = io.nev0, np0 = io.np0, nconv = io.nconv;
    std::vector<double> rz(io.ritz_s, io.ritz_s + m), bix(m), d(m), e(m), Z((size_t)m * m), tau(m, 0.0);
    std::vector<char> sel(m, 0);
    for (int j = 0; j < m; ++j) bix[j] = j + 1;
    dsgets(nev0, np0, rz.data(), bix.data());            // HLanc.hpp:1768-1793
    int numcnv = 0;
    for (int j = 0; j < m; ++j) {
        const double temp1 = fmax(io.eps23, fabs(rz[m - j - 1]));
        const int jj = (int)bix[m - j - 1];
        if (numcnv < nconv && io.bnds_s[jj - 1] <= io.tol * temp1) {
            sel[jj - 1] = 1;
            ++numcnv;
        }
    }
    if (numcnv != nconv) return 1;
    for (int i = 0; i < m; ++i) {
        d[i] = io.h[m + i];
        e[i] = (i + 1 < m) ? io.h[i + 1] : 0.0;
    }
    if (tridiag_eig(m, d.data(), e.data(), nullptr, Z.data(), m)) return 1;   // HLanc.hpp:1805
    auto swapcol = [&](int a, int b) {
        for (int i = 0; i < m; ++i) std::swap(Z[i + (size_t)a * m], Z[i + (size_t)b * m]);
    };
    int left = 0, right = m - 1;                          // HLanc.hpp:1808-1831
    for (;;) {
        while (left < m && sel[left]) ++left;
        while (right >= 0 && !sel[right]) --right;
        if (left > right) break;
        std::swap(d[left], d[right]);
        swapcol(left, right);
        ++left; --right;
    }
    std::vector<int> idx(nconv);                          // dsesrt, HLanc.hpp:1626-1647
    for (int i = 0; i < nconv; ++i) idx[i] = i;
    for (int i = 1; i < nconv; ++i) {
        const int x = idx[i];
        int j = i - 1;
        while (j >= 0 && d[x] < d[idx[j]]) { idx[j + 1] = idx[j]; --j; }
        idx[j + 1] = x;
    }
    std::vector<double> Zs((size_t)m * nconv);
    for (int c = 0; c < nconv; ++c) {
        io.values[c] = d[idx[c]];
        memcpy(&Zs[(size_t)c * m], &Z[(size_t)idx[c] * m], sizeof(double) * m);
    }
    memcpy(Z.data(), Zs.data(), sizeof(double) * (size_t)m * nconv);
    // Householder QR of Z[:, 0:nconv) (dgeqr2, HLanc.hpp:1837)
    for (int i = 0; i < nconv; ++i) {
        double *col = &Z[i + (size_t)i * m];
        const int len = m - i;
        const double alpha = col[0];
        double xn = 0.0;
        for (int t = 1; t < len; ++t) xn = hypot(xn, col[t]);
        if (xn == 0.0) { tau[i] = 0.0; continue; }
        const double beta = -copysign(hypot(alpha, xn), alpha);
        tau[i] = (beta - alpha) / beta;
        const double scal = 1.0 / (alpha - beta);
        for (int t = 1; t < len; ++t) col[t] *= scal;
        col[0] = beta;
        for (int jc = i + 1; jc < nconv; ++jc) {
            double *cj = &Z[i + (size_t)jc * m];
            double w = cj[0];
            for (int t = 1; t < len; ++t) w += col[t] * cj[t];
            w *= tau[i];
            cj[0] -= w;
            for (int t = 1; t < len; ++t) cj[t] -= w * col[t];
        }
    }
    // Q2 = H_0 H_1 ... H_{nconv-1}: the factor dorm2r applies (HLanc.hpp:1840)
    double *Q2 = io.Q2;
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) Q2[i + (size_t)j * m] = (i == j) ? 1.0 : 0.0;
    for (int i = 0; i < nconv; ++i) {
        if (tau[i] == 0.0) continue;
        const double *v = &Z[i + (size_t)i * m];
        for (int r = 0; r < m; ++r) {
            double w = Q2[r + (size_t)i * m];
            for (int t = 1; t < m - i; ++t) w += Q2[r + (size_t)(i + t) * m] * v[t];
            w *= tau[i];
            Q2[r + (size_t)i * m] -= w;
            for (int t = 1; t < m - i; ++t) Q2[r + (size_t)(i + t) * m] -= w * v[t];
        }
    }
    return 0;
}

}  // namespace host
}  // namespace hlanc
