// kernels_restart.cu -- restart cycle and post-processing on the device
//
//   k_restart   one CTA per problem: Ritz values and last eigenvector
//               components of T (replaces dsteqr, HLanc.hpp:1691), bounds,
//               dsgets / dsconv / nev-np adjustment (HLanc.hpp:1693-1730) and
//               the implicit shifted-QR Givens chain of dsapps
//               (HLanc.hpp:1485-1589), accumulating Q in HBM.
//   k_basis     V <- V Q[:, 0:nev] and the new residual (HLanc.hpp:1591-1614)
//               in one pass over V (replaces nev GEMVs + kernel_move_columns).
//   k_finalize  one CTA per converged problem: select/reorder/sort the
//               converged Ritz pairs, eigenvectors of T, Householder QR of the
//               selected eigenvectors and the explicit orthogonal factor
//               (HLanc.hpp:1765-1842).
//   k_ritz      vectors = V Qfull in one pass over V (replaces the per-
//               reflector gemv+ger of mat_v_gpu_t::dorm2r_RN, HLanc.hpp:1075-1107)
//               on the FP64 CUDA cores; the tensor-core form (kernels_tc.cu)
//               is the default for ncv <= 64.
//
// Small dense algorithms are written from their textbook definitions:
// tridiagonal QR with Wilkinson shift (Golub & Van Loan 4e, Alg. 8.3.2/8.3.3),
// Givens generation with the LAPACK >= 3.10 convention (c >= 0, r signed like
// f; Anderson, ACM TOMS 2017), Householder QR (Golub & Van Loan Alg. 5.1.1).
// Sequential scalar work runs on thread 0 of the CTA; every update of a dense
// ncv x ncv matrix is applied row-parallel by the CTA's threads.
#include <float.h>

#include "internal.cuh"

namespace hlanc {

constexpr int RTPB = 128;   // threads of the per-problem CTAs (>= MAXNCV)

__device__ void dev_givens(double f, double g, double &c, double &s, double &r) {
    if (g == 0.0) { c = 1.0; s = 0.0; r = f; return; }
    if (f == 0.0) { c = 0.0; s = copysign(1.0, g); r = fabs(g); return; }
    const double f1 = fabs(f), g1 = fabs(g);
    const double rtmin = 1.4916681462400413e-154;   // sqrt(DBL_MIN)
    const double rtmax = 9.4807519081091774e+153;   // sqrt(DBL_MAX / 2)
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

// Symmetric tridiagonal eigensolver, CTA-cooperative.  d[n], e[n-1] in
// shared memory; zl (shared, optional) is the last row of the eigenvector
// matrix, updated by thread 0; Z (global, optional, n x n, ldz) receives the
// eigenvectors, rotated row-parallel after each sweep.  Eigenvalues ascending
// (selection sort, columns swapped alike).  Returns nonzero on failure.
__device__ int cta_tridiag_eig(int n, double *d, double *e, double *zl, double *Z, int ldz,
                               double *rot_c, double *rot_s, int *sint, int *swaps) {
    const int tid = threadIdx.x;
    if (Z)
        for (int idx = tid; idx < n * n; idx += blockDim.x) {
            const int i = idx % n, jj = idx / n;
            Z[i + (size_t)jj * ldz] = (i == jj) ? 1.0 : 0.0;
        }
    if (tid == 0) { sint[0] = n - 1; sint[1] = -1; sint[2] = 0; sint[3] = 0; }
    __syncthreads();
    const double eps = DBL_EPSILON * 0.5;
    for (;;) {
        if (tid == 0) {
            int hi = sint[0], lo = -1;
            if (hi > 0) {
                for (int i = 0; i < hi; ++i)
                    if (fabs(e[i]) <= eps * (fabs(d[i]) + fabs(d[i + 1])) || fabs(e[i]) < DBL_MIN) e[i] = 0.0;
                while (hi > 0 && e[hi - 1] == 0.0) --hi;
                if (hi > 0) {
                    lo = hi - 1;
                    while (lo > 0 && e[lo - 1] != 0.0) --lo;
                    if (++sint[2] > 30 * n) {
                        sint[3] = 1;
                        lo = -1;
                        hi = 0;
                    } else {
                        const double dd = 0.5 * (d[hi - 1] - d[hi]);
                        const double b = e[hi - 1];
                        const double den = dd + copysign(hypot(dd, b), dd);
                        const double mu = (den != 0.0) ? d[hi] - b * (b / den) : d[hi] - fabs(b);
                        double x = d[lo] - mu, zz = e[lo];
                        for (int k = lo; k < hi; ++k) {
                            const double r = hypot(x, zz);
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
                            rot_c[k] = c;
                            rot_s[k] = s;
                            if (zl) {
                                const double a0 = zl[k], a1 = zl[k + 1];
                                zl[k] = c * a0 + s * a1;
                                zl[k + 1] = -s * a0 + c * a1;
                            }
                        }
                    }
                }
            }
            sint[0] = hi;
            sint[1] = lo;
        }
        __syncthreads();
        const int lo = sint[1], hi = sint[0];
        if (lo < 0) break;
        if (Z && tid < n) {
            double *zr = Z + tid;
            for (int k = lo; k < hi; ++k) {
                const double c = rot_c[k], s = rot_s[k];
                const double a0 = zr[(size_t)k * ldz], a1 = zr[(size_t)(k + 1) * ldz];
                zr[(size_t)k * ldz] = c * a0 + s * a1;
                zr[(size_t)(k + 1) * ldz] = -s * a0 + c * a1;
            }
        }
        __syncthreads();
    }
    // ascending order by selection sort; the swaps are replayed on Z's rows
    if (tid == 0) {
        int ns = 0;
        for (int i = 0; i < n - 1; ++i) {
            int k = i;
            for (int jj = i + 1; jj < n; ++jj)
                if (d[jj] < d[k]) k = jj;
            if (k != i) {
                const double t = d[i]; d[i] = d[k]; d[k] = t;
                if (zl) { const double tz = zl[i]; zl[i] = zl[k]; zl[k] = tz; }
                swaps[2 * ns] = i;
                swaps[2 * ns + 1] = k;
                ++ns;
            }
        }
        sint[2] = ns;
    }
    __syncthreads();
    if (Z && tid < n) {
        double *zr = Z + tid;
        for (int q = 0; q < sint[2]; ++q) {
            const int a = swaps[2 * q], b = swaps[2 * q + 1];
            const double t = zr[(size_t)a * ldz];
            zr[(size_t)a * ldz] = zr[(size_t)b * ldz];
            zr[(size_t)b * ldz] = t;
        }
    }
    const int fail = sint[3];
    __syncthreads();
    return fail;
}

// dsgets (HLanc.hpp:1387-1401): sort by Ritz value ascending, then the first
// np by bound descending.  Stable insertion sorts (thread 0).
__device__ void dev_dsgets(int nev, int np, double *ritz, double *bounds) {
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

// ---- the restart kernel ---------------------------------------------------------
__global__ void __launch_bounds__(RTPB) k_restart(const Problem *__restrict__ probs) {
    const Problem &P = probs[blockIdx.x];
    State *S = P.st;
    if (S->status != ST_RUNNING || S->phase != PH_EXTEND || S->iter < 0) return;
    const int m = P.ncv, tid = threadIdx.x;
    double *sm = P.small;
    double *h = sm + SM_H(m);
    double *ritz = sm + SM_RITZ(m);
    double *bounds = sm + SM_BOUNDS(m);
    double *Q = sm + SM_Q(m);
    __shared__ double d[MAXNCV], e[MAXNCV], zl[MAXNCV], rc[MAXNCV], rs[MAXNCV];
    __shared__ int sint[8];
    __shared__ int swaps[2 * MAXNCV];
    __shared__ int s_go, s_nev, s_np, s_itop, s_nops;
    __shared__ double op_c[2 * MAXNCV], op_s[2 * MAXNCV];
    __shared__ int op_col[2 * MAXNCV], op_lim[2 * MAXNCV];

    for (int i = tid; i < m; i += blockDim.x) {
        d[i] = h[m + i];
        e[i] = (i + 1 < m) ? h[i + 1] : 0.0;
        zl[i] = (i == m - 1) ? 1.0 : 0.0;
    }
    __syncthreads();
    const int fail = cta_tridiag_eig(m, d, e, zl, nullptr, 0, rc, rs, sint, swaps);
    if (tid == 0) {
        S->iter += 1;
        s_go = 0;
        if (fail) {
            S->status = ST_FAILED;        // dsteqr info != 0 -> return 1 (HLanc.hpp:1692)
            S->phase = PH_DONE;
        } else {
            const double rnorm = S->rnorm;
            for (int i = 0; i < m; ++i) {
                ritz[i] = d[i];
                bounds[i] = rnorm * fabs(zl[i]);                    // HLanc.hpp:1693-1695
                sm[SM_RITZS(m) + i] = ritz[i];                      // HLanc.hpp:1697-1698
                sm[SM_BNDS(m) + i] = bounds[i];
            }
            int nev = S->nev0, np = S->np0;
            dev_dsgets(nev, np, ritz, bounds);
            int nconv = 0;                                           // dsconv, HLanc.hpp:1377-1384
            for (int i = 0; i < nev; ++i)
                nconv += bounds[np + i] <= S->tol * fmax(S->eps23, fabs(ritz[np + i]));
            for (int jj = 0; jj < np; ++jj)                          // HLanc.hpp:1708-1713
                if (bounds[jj] == 0.0) { --np; ++nev; }
            S->nconv = nconv;
            if (nconv >= S->nev0 || np == 0) {
                S->status = (nconv >= S->nev0) ? ST_CONVERGED : ST_NOT_CONVERGED;
                S->phase = PH_DONE;
            } else if (S->iter >= S->max_iter) {
                S->status = ST_NOT_CONVERGED;                        // HLanc.hpp:1762
                S->phase = PH_DONE;
            } else {
                const int nevbef = nev;                              // HLanc.hpp:1719-1730
                nev += (nconv < np / 2) ? nconv : np / 2;
                if (nev == 1 && m >= 6) nev = m / 2;
                else if (nev == 1 && m > 2) nev = 2;
                np = m - nev;
                if (nevbef < nev) dev_dsgets(nev, np, ritz, bounds);
                s_go = 1;
                s_nev = nev;
                s_np = np;
            }
        }
    }
    __syncthreads();
    if (!s_go) return;
    const int nev = s_nev, np = s_np;
    // ---- dsapps (HLanc.hpp:1485-1589) ----
    for (int idx = tid; idx < m * m; idx += blockDim.x) Q[idx] = (idx % m == idx / m) ? 1.0 : 0.0;
    if (tid == 0) s_itop = 1;
    __syncthreads();
    const double epsmch = DBL_EPSILON * 0.5;
    for (int jj = 1; jj <= np; ++jj) {
        if (tid == 0) {
            int nops = 0;
            int itop = s_itop;
            int istart = itop;
            double c = 0.0, s = 0.0, r = 0.0;
            for (;;) {
                int iend = m;
                for (int i = istart; i <= m - 1; ++i) {
                    const double big = fabs(h[m + i - 1]) + fabs(h[m + i]);
                    if (h[i] <= epsmch * big) { h[i] = 0.0; iend = i; break; }
                }
                if (istart < iend) {
                    double f = h[istart + m - 1] - ritz[jj - 1];
                    double g = h[istart];
                    dev_givens(f, g, c, s, r);
                    const double a1 = c * h[istart + m - 1] + s * h[istart];
                    const double a2 = c * h[istart] + s * h[istart + m];
                    const double a4 = c * h[istart + m] - s * h[istart];
                    const double a3 = c * h[istart] - s * h[istart + m - 1];
                    h[istart + m - 1] = c * a1 + s * a2;
                    h[istart + m] = c * a4 - s * a3;
                    h[istart] = c * a3 + s * a4;
                    op_col[nops] = istart;
                    op_lim[nops] = (istart + jj < m) ? istart + jj : m;
                    op_c[nops] = c; op_s[nops] = s; ++nops;
                    for (int i = istart + 1; i <= iend - 1; ++i) {
                        f = h[i - 1];
                        g = s * h[i];
                        h[i] = c * h[i];
                        dev_givens(f, g, c, s, r);
                        if (r < 0.0) { r = -r; c = -c; s = -s; }
                        h[i - 1] = r;
                        const double b1 = c * h[i + m - 1] + s * h[i];
                        const double b2 = c * h[i] + s * h[i + m];
                        const double b3 = c * h[i] - s * h[i + m - 1];
                        const double b4 = c * h[i + m] - s * h[i];
                        h[i + m - 1] = c * b1 + s * b2;
                        h[i + m] = c * b4 - s * b3;
                        h[i] = c * b3 + s * b4;
                        op_col[nops] = i;
                        op_lim[nops] = (i + jj < m) ? i + jj : m;
                        op_c[nops] = c; op_s[nops] = s; ++nops;
                    }
                }
                istart = iend + 1;
                if (h[iend - 1] < 0.0) {
                    h[iend - 1] = -h[iend - 1];
                    op_col[nops] = iend - 1;
                    op_lim[nops] = -1;               // negate column
                    op_c[nops] = 0.0; op_s[nops] = 0.0; ++nops;
                }
                if (iend < m) continue;
                for (int i = itop; i <= m - 1; ++i) {
                    if (h[i] > 0.0) break;
                    ++itop;
                }
                break;
            }
            s_itop = itop;
            s_nops = nops;
        }
        __syncthreads();
        if (tid < m) {
            double *qr = Q + tid;
            const int nops = s_nops;
            for (int q = 0; q < nops; ++q) {
                const int col = op_col[q], lim = op_lim[q];
                if (lim < 0) {
                    qr[(size_t)col * m] = -qr[(size_t)col * m];
                } else if (tid < lim) {
                    const double c = op_c[q], s = op_s[q];
                    const double a = qr[(size_t)(col - 1) * m], b = qr[(size_t)col * m];
                    qr[(size_t)(col - 1) * m] = c * a + s * b;
                    qr[(size_t)col * m] = -s * a + c * b;
                }
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        for (int i = s_itop; i <= m - 1; ++i) {                       // HLanc.hpp:1584-1589
            const double big = fabs(h[i + m - 1]) + fabs(h[i + m]);
            if (h[i] <= epsmch * big) h[i] = 0.0;
        }
        S->nev = nev;
        S->np = np;
        S->k = nev;
        S->phase = PH_APPLY;
    }
}

// ---- basis update: V[:, 0:nev) <- V Q[:, 0:nev), new residual ---------------
// Thread per row.  Q[k, i] = 0 for k > i + np (np shifts keep Q banded), so
// only the band is multiplied.  Each thread reads its whole row of V before
// writing, so the update is in place.
template <int MAXOUT>
__global__ void __launch_bounds__(TPB) k_basis(const Problem *__restrict__ probs,
                                               const Tile *__restrict__ tiles) {
    const Tile t = tiles[blockIdx.x];
    const Problem &P = probs[t.prob];
    State *S = P.st;
    if (S->status != ST_RUNNING || S->phase != PH_APPLY) return;
    const int m = P.ncv, nev = S->nev, np = S->np;
    extern __shared__ double qs[];                 // m x (MAXOUT + 1): columns 0..MAXOUT-1, then column nev
    const double *Q = P.small + SM_Q(m);
    const double *h = P.small + SM_H(m);
    for (int idx = threadIdx.x; idx < m * (MAXOUT + 1); idx += TPB) {
        const int k = idx / (MAXOUT + 1), i = idx % (MAXOUT + 1);
        double q = 0.0;
        if (i < MAXOUT) { if (i < nev && k <= i + np) q = Q[k + (size_t)i * m]; }
        else q = Q[k + (size_t)nev * m];
        qs[idx] = q;
    }
    __shared__ double scratch[32], mine[1], tot[1];
    __syncthreads();
    const double hn = h[nev];
    const double qlast = Q[(m - 1) + (size_t)(nev - 1) * m];
    const double *__restrict__ rin = (m & 1) ? P.r1 : P.r0;
    double *__restrict__ rout = (nev & 1) ? P.r1 : P.r0;
    const size_t ld = (size_t)P.ld;
    double nrm = 0.0;
    for (int r = t.row0 + threadIdx.x; r < t.row1; r += TPB) {
        double acc[MAXOUT];
#pragma unroll
        for (int i = 0; i < MAXOUT; ++i) acc[i] = 0.0;
        double accn = 0.0;
        double *vr = P.V + r;
        for (int k = 0; k < m; ++k) {
            const double v = vr[(size_t)k * ld];
            const double *qk = qs + k * (MAXOUT + 1);
            const int i0 = k - np;                  // first output column whose band reaches k
#pragma unroll
            for (int i = 0; i < MAXOUT; ++i)
                if (i >= i0 && i < nev) acc[i] = fma(v, qk[i], acc[i]);
            accn = fma(v, qk[MAXOUT], accn);
        }
        float *vr32 = P.V32 + r;
#pragma unroll
        for (int i = 0; i < MAXOUT; ++i)
            if (i < nev) {
                vr[(size_t)i * ld] = acc[i];
                vr32[(size_t)i * ld] = (float)acc[i];
            }
        double res = rin[r] * qlast;                // HLanc.hpp:1605-1614
        if (hn > 0.0) res = res + hn * accn;
        rout[r] = res;
        nrm = fma(res, res, nrm);
    }
    nrm = block_sum0(nrm, scratch);
    if (threadIdx.x == 0) mine[0] = nrm;
    __syncthreads();
    if (!finish_tile(P, blockIdx.x - P.tile0, 1, mine, tot)) return;
    if (threadIdx.x == 0) {
        S->rnorm = sqrt(tot[0]);                    // HLanc.hpp:1735
        S->phase = PH_EXTEND;
        S->sumnev += nev;
        S->napply += 1;
    }
}

// The same update when the adjusted nev exceeds the 64 outputs k_basis and
// k_basis_tc hold (possible for ncv > 64: nev grows by up to half of np).
// The update is in place and every output reads every column of the row, so
// each thread first copies its row of V to shared memory (64 threads per
// CTA, a row of up to 128 columns each), then writes the outputs in order.
// The sums run over k in ascending order with the same band as k_basis, so
// the results are the same.
constexpr int WIDE_TPB = 64;
__global__ void __launch_bounds__(WIDE_TPB) k_basis_wide(const Problem *__restrict__ probs,
                                                         const Tile *__restrict__ tiles) {
    const Tile t = tiles[blockIdx.x];
    const Problem &P = probs[t.prob];
    State *S = P.st;
    if (S->status != ST_RUNNING || S->phase != PH_APPLY) return;
    const int m = P.ncv, nev = S->nev, np = S->np;
    extern __shared__ double rows[];               // WIDE_TPB x (m + 1): each thread's row
    const double *Q = P.small + SM_Q(m);
    const double *h = P.small + SM_H(m);
    __shared__ double scratch[32], mine[1], tot[1];
    const double hn = h[nev];
    const double qlast = Q[(m - 1) + (size_t)(nev - 1) * m];
    const double *__restrict__ rin = (m & 1) ? P.r1 : P.r0;
    double *__restrict__ rout = (nev & 1) ? P.r1 : P.r0;
    const size_t ld = (size_t)P.ld;
    double *my = rows + (size_t)threadIdx.x * (m + 1);
    double nrm = 0.0;
    for (int r = t.row0 + threadIdx.x; r < t.row1; r += WIDE_TPB) {
        double *vr = P.V + r;
        for (int k = 0; k < m; ++k) my[k] = vr[(size_t)k * ld];
        for (int i = 0; i < nev; ++i) {
            const int k1 = min(m, i + np + 1);     // band of output i: k <= i + np
            const double *qi = Q + (size_t)i * m;
            double acc = 0.0;
            for (int k = 0; k < k1; ++k) acc = fma(my[k], qi[k], acc);
            vr[(size_t)i * ld] = acc;
            P.V32[r + (size_t)i * ld] = (float)acc;
        }
        const double *qn = Q + (size_t)nev * m;
        double accn = 0.0;
        for (int k = 0; k < m; ++k) accn = fma(my[k], qn[k], accn);
        double res = rin[r] * qlast;                // HLanc.hpp:1605-1614
        if (hn > 0.0) res = res + hn * accn;
        rout[r] = res;
        nrm = fma(res, res, nrm);
    }
    nrm = block_sum0(nrm, scratch);
    if (threadIdx.x == 0) mine[0] = nrm;
    __syncthreads();
    if (!finish_tile(P, blockIdx.x - P.tile0, 1, mine, tot)) return;
    if (threadIdx.x == 0) {
        S->rnorm = sqrt(tot[0]);                    // HLanc.hpp:1735
        S->phase = PH_EXTEND;
        S->sumnev += nev;
        S->napply += 1;
    }
}

// ---- finalize: converged Ritz pairs (HLanc.hpp:1765-1842) -------------------
__global__ void __launch_bounds__(RTPB) k_finalize(const Problem *__restrict__ probs) {
    const Problem &P = probs[blockIdx.x];
    State *S = P.st;
    if (S->status != ST_CONVERGED || S->fin != 0) return;
    const int m = P.ncv, tid = threadIdx.x;
    const int nev0 = S->nev0, np0 = S->np0, nconv = S->nconv;
    double *sm = P.small;
    const double *h = sm + SM_H(m);
    double *Z = sm + SM_Q(m);       // eigenvectors of T, then Householder vectors
    double *Q2 = sm + SM_Q2(m);     // explicit orthogonal factor
    double *vals = sm + SM_VALS(m);
    __shared__ double rz[MAXNCV], bix[MAXNCV], d[MAXNCV], e[MAXNCV], rc[MAXNCV], rs[MAXNCV];
    __shared__ double tau[MAXNCV];
    __shared__ int sel[MAXNCV], sint[8], swaps[4 * MAXNCV], idx[MAXNCV], pos[MAXNCV];
    __shared__ int s_ok, s_nsw;
    __shared__ double s_scal, s_beta;
    if (tid == 0) {
        // selection of the converged pairs (HLanc.hpp:1768-1793)
        for (int jq = 0; jq < m; ++jq) { rz[jq] = sm[SM_RITZS(m) + jq]; bix[jq] = jq + 1; sel[jq] = 0; }
        dev_dsgets(nev0, np0, rz, bix);
        int numcnv = 0;
        for (int jq = 0; jq < m; ++jq) {
            const double temp1 = fmax(S->eps23, fabs(rz[m - jq - 1]));
            const int jj = (int)bix[m - jq - 1];
            if (numcnv < nconv && sm[SM_BNDS(m) + jj - 1] <= S->tol * temp1) {
                sel[jj - 1] = 1;
                ++numcnv;
            }
        }
        s_ok = (numcnv == nconv);
    }
    for (int i = tid; i < m; i += blockDim.x) {
        d[i] = h[m + i];
        e[i] = (i + 1 < m) ? h[i + 1] : 0.0;
    }
    __syncthreads();
    if (!s_ok) {
        if (tid == 0) { S->status = ST_FAILED; S->fin = 2; }
        return;
    }
    if (cta_tridiag_eig(m, d, e, nullptr, Z, m, rc, rs, sint, swaps)) {
        if (tid == 0) { S->status = ST_FAILED; S->fin = 2; }
        return;
    }
    // move the selected pairs to the front (HLanc.hpp:1808-1831)
    if (tid == 0) {
        int ns = 0, left = 0, right = m - 1;
        for (;;) {
            while (left < m && sel[left]) ++left;
            while (right >= 0 && !sel[right]) --right;
            if (left > right) break;
            const double t = d[left]; d[left] = d[right]; d[right] = t;
            swaps[2 * ns] = left; swaps[2 * ns + 1] = right; ++ns;
            ++left; --right;
        }
        // dsesrt (HLanc.hpp:1626-1647): stable ascending order of the first nconv
        for (int i = 0; i < nconv; ++i) idx[i] = i;
        for (int i = 1; i < nconv; ++i) {
            const int x = idx[i];
            int jq = i - 1;
            while (jq >= 0 && d[x] < d[idx[jq]]) { idx[jq + 1] = idx[jq]; --jq; }
            idx[jq + 1] = x;
        }
        for (int i = 0; i < nconv; ++i) rz[i] = d[idx[i]];
        for (int i = 0; i < nconv; ++i) { d[i] = rz[i]; vals[i] = rz[i]; }
        // the column permutation new[c] = old[idx[c]] as a swap list
        for (int i = 0; i < m; ++i) pos[i] = i;        // pos[slot] = original column held there
        for (int c = 0; c < nconv; ++c) {
            int p = c;
            while (pos[p] != idx[c]) ++p;
            if (p != c) {
                swaps[2 * ns] = c; swaps[2 * ns + 1] = p; ++ns;
                const int t = pos[c]; pos[c] = pos[p]; pos[p] = t;
            }
        }
        s_nsw = ns;
    }
    __syncthreads();
    if (tid < m) {
        double *zr = Z + tid;
        for (int q = 0; q < s_nsw; ++q) {
            const int a = swaps[2 * q], b = swaps[2 * q + 1];
            const double t = zr[(size_t)a * m];
            zr[(size_t)a * m] = zr[(size_t)b * m];
            zr[(size_t)b * m] = t;
        }
    }
    __syncthreads();
    // Householder QR of Z[:, 0:nconv) (dgeqr2, HLanc.hpp:1837)
    for (int i = 0; i < nconv; ++i) {
        double *col = Z + i + (size_t)i * m;
        const int len = m - i;
        if (tid == 0) {
            const double alpha = col[0];
            double xn = 0.0;
            for (int t = 1; t < len; ++t) xn = hypot(xn, col[t]);
            if (xn == 0.0) {
                tau[i] = 0.0; s_scal = 1.0; s_beta = alpha;
            } else {
                const double beta = -copysign(hypot(alpha, xn), alpha);
                tau[i] = (beta - alpha) / beta;
                s_scal = 1.0 / (alpha - beta);
                s_beta = beta;
            }
        }
        __syncthreads();
        if (tau[i] != 0.0) {
            for (int t = 1 + tid; t < len; t += blockDim.x) col[t] *= s_scal;
            __syncthreads();
            if (tid == 0) col[0] = s_beta;
            for (int jc = i + 1 + tid; jc < nconv; jc += blockDim.x) {
                double *cj = Z + i + (size_t)jc * m;
                double w = cj[0];
                for (int t = 1; t < len; ++t) w += col[t] * cj[t];
                w *= tau[i];
                cj[0] -= w;
                for (int t = 1; t < len; ++t) cj[t] -= w * col[t];
            }
        }
        __syncthreads();
    }
    // Q2 = H_0 H_1 ... H_{nconv-1} (the factor dorm2r applies, HLanc.hpp:1840)
    if (tid < m) {
        double *qr = Q2 + tid;
        for (int c = 0; c < m; ++c) qr[(size_t)c * m] = (c == tid) ? 1.0 : 0.0;
        for (int i = 0; i < nconv; ++i) {
            if (tau[i] == 0.0) continue;
            const double *v = Z + i + (size_t)i * m;
            double w = qr[(size_t)i * m];
            for (int t = 1; t < m - i; ++t) w += qr[(size_t)(i + t) * m] * v[t];
            w *= tau[i];
            qr[(size_t)i * m] -= w;
            for (int t = 1; t < m - i; ++t) qr[(size_t)(i + t) * m] -= w * v[t];
        }
    }
    __syncthreads();
    if (tid == 0) S->fin = 1;
}

// ---- Ritz vectors: out = V Q2 (all ncv columns, HLanc.hpp:1840-1843) -------------
constexpr int RITZ_PANEL = 32;
__global__ void __launch_bounds__(TPB) k_ritz(const Problem *__restrict__ probs,
                                              const Tile *__restrict__ tiles) {
    const Tile t = tiles[blockIdx.x];
    const Problem &P = probs[t.prob];
    State *S = P.st;
    if (S->status != ST_CONVERGED || S->fin != 1) return;
    const int m = P.ncv;
    const double *Q2 = P.small + SM_Q2(m);
    extern __shared__ double qs[];                  // m x RITZ_PANEL
    const size_t ld = (size_t)P.ld, ldo = (size_t)P.ldo;
    for (int p0 = 0; p0 < m; p0 += RITZ_PANEL) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < m * RITZ_PANEL; idx += TPB) {
            const int k = idx / RITZ_PANEL, i = idx % RITZ_PANEL;
            qs[idx] = (p0 + i < m) ? Q2[k + (size_t)(p0 + i) * m] : 0.0;
        }
        __syncthreads();
        for (int r = t.row0 + threadIdx.x; r < t.row1; r += TPB) {
            double acc[RITZ_PANEL];
#pragma unroll
            for (int i = 0; i < RITZ_PANEL; ++i) acc[i] = 0.0;
            const double *vr = P.V + r;
            for (int k = 0; k < m; ++k) {
                const double v = vr[(size_t)k * ld];
                const double *qk = qs + k * RITZ_PANEL;
#pragma unroll
                for (int i = 0; i < RITZ_PANEL; ++i) acc[i] = fma(v, qk[i], acc[i]);
            }
#pragma unroll
            for (int i = 0; i < RITZ_PANEL; ++i)
                if (p0 + i < m) P.vout[(size_t)(p0 + i) * ldo + r] = acc[i];
        }
    }
    __shared__ double mine[1], tot[1];
    if (threadIdx.x == 0) mine[0] = 0.0;
    __syncthreads();
    if (!finish_tile(P, blockIdx.x - P.tile0, 1, mine, tot)) return;
    if (threadIdx.x == 0) S->fin = 2;
}

// ---- host-restart mailbox: one gather / one scatter per cycle -----------------
// Per problem a, at off[a] (doubles): [State (32 doubles) | h (2m) | Q (m*m) | values (m)].
static_assert(sizeof(State) <= 32 * sizeof(double), "State must fit its mailbox slot");

__global__ void k_gather(const Problem *__restrict__ probs, const long long *__restrict__ off,
                         double *__restrict__ buf) {
    const Problem &P = probs[blockIdx.x];
    double *o = buf + off[blockIdx.x];
    const double *st = reinterpret_cast<const double *>(P.st);
    const int ns = (int)(sizeof(State) / sizeof(double));
    for (int i = threadIdx.x; i < ns; i += blockDim.x) o[i] = st[i];
    for (int i = threadIdx.x; i < 2 * P.ncv; i += blockDim.x) o[32 + i] = P.small[SM_H(P.ncv) + i];
}

// flag 1: State + h + Q (a restart to apply); 2: State only; 3: State + Q2 +
// values (finalised pair set); 0: nothing.
__global__ void k_scatter(const Problem *__restrict__ probs, const long long *__restrict__ off,
                          const int *__restrict__ flag, const double *__restrict__ buf) {
    const int f = flag[blockIdx.x];
    if (!f) return;
    const Problem &P = probs[blockIdx.x];
    const int m = P.ncv;
    const double *in = buf + off[blockIdx.x];
    double *st = reinterpret_cast<double *>(P.st);
    const int ns = (int)(sizeof(State) / sizeof(double));
    for (int i = threadIdx.x; i < ns; i += blockDim.x) st[i] = in[i];
    if (f == 1) {
        for (int i = threadIdx.x; i < 2 * m; i += blockDim.x) P.small[SM_H(m) + i] = in[32 + i];
        for (int i = threadIdx.x; i < m * m; i += blockDim.x) P.small[SM_Q(m) + i] = in[32 + 2 * m + i];
    } else if (f == 3) {
        for (int i = threadIdx.x; i < m * m; i += blockDim.x) P.small[SM_Q2(m) + i] = in[32 + 2 * m + i];
        for (int i = threadIdx.x; i < m; i += blockDim.x) P.small[SM_VALS(m) + i] = in[32 + 2 * m + m * m + i];
    }
}

// ---- launchers -------------------------------------------------------------------
void launch_gather(const Problem *P_d, int nprob, const long long *off_d, double *buf_d, cudaStream_t s) {
    prof_begin(s);
    k_gather<<<nprob, 128, 0, s>>>(P_d, off_d, buf_d);
    prof_end(KC_AUX, s);
    launch_counter() += 1;
}

void launch_scatter(const Problem *P_d, int nprob, const long long *off_d, const int *flag_d,
                    const double *buf_d, cudaStream_t s) {
    prof_begin(s);
    k_scatter<<<nprob, 256, 0, s>>>(P_d, off_d, flag_d, buf_d);
    prof_end(KC_AUX, s);
    launch_counter() += 1;
}

void launch_restart(const Problem *P_d, int nprob, int, cudaStream_t s) {
    prof_begin(s);
    k_restart<<<nprob, RTPB, 0, s>>>(P_d);
    prof_end(KC_AUX, s);
    launch_counter() += 1;
}

template <int MAXOUT>
static void basis_t(const Problem *P_d, const Tile *tiles_d, int ntiles, int max_ncv, cudaStream_t s) {
    const size_t smem = sizeof(double) * (size_t)max_ncv * (MAXOUT + 1);
    static std::atomic<unsigned long long> attr{0};
    smem_limit_once(k_basis<MAXOUT>, 160 * 1024, attr);
    prof_begin(s);
    k_basis<MAXOUT><<<ntiles, TPB, smem, s>>>(P_d, tiles_d);
    prof_end(KC_BASIS, s);
}

// nev is rounded up to a multiple of 4: the unrolled output loop issues no
// FP64 instruction for more than 3 absent columns.
void launch_basis(const Problem *P_d, const Tile *tiles_d, int ntiles, int max_ncv, int max_nev,
                  bool tensor_cores, cudaStream_t s) {
    if (tensor_cores && basis_tc_fits(max_ncv, max_nev)) {
        launch_basis_tc(P_d, tiles_d, ntiles, max_nev, s);
        return;
    }
    if (max_nev > 64) {
        const size_t smem = sizeof(double) * (size_t)WIDE_TPB * (max_ncv + 1);
        static std::atomic<unsigned long long> attr{0};
        smem_limit_once(k_basis_wide, (int)(sizeof(double) * WIDE_TPB * (MAXNCV + 1)), attr);
        prof_begin(s);
        k_basis_wide<<<ntiles, WIDE_TPB, smem, s>>>(P_d, tiles_d);
        prof_end(KC_BASIS, s);
        launch_counter() += 1;
        variant_counter(HLANC_KL_BASIS_FP64) += 1;
        return;
    }
    switch ((max_nev + 3) / 4) {
    case 0: case 1: basis_t<4>(P_d, tiles_d, ntiles, max_ncv, s); break;
    case 2: basis_t<8>(P_d, tiles_d, ntiles, max_ncv, s); break;
    case 3: basis_t<12>(P_d, tiles_d, ntiles, max_ncv, s); break;
    case 4: basis_t<16>(P_d, tiles_d, ntiles, max_ncv, s); break;
    case 5: basis_t<20>(P_d, tiles_d, ntiles, max_ncv, s); break;
    case 6: basis_t<24>(P_d, tiles_d, ntiles, max_ncv, s); break;
    case 7: basis_t<28>(P_d, tiles_d, ntiles, max_ncv, s); break;
    case 8: basis_t<32>(P_d, tiles_d, ntiles, max_ncv, s); break;
    case 9: basis_t<36>(P_d, tiles_d, ntiles, max_ncv, s); break;
    case 10: basis_t<40>(P_d, tiles_d, ntiles, max_ncv, s); break;
    case 11: case 12: basis_t<48>(P_d, tiles_d, ntiles, max_ncv, s); break;
    case 13: case 14: basis_t<56>(P_d, tiles_d, ntiles, max_ncv, s); break;
    default: basis_t<64>(P_d, tiles_d, ntiles, max_ncv, s); break;
    }
    launch_counter() += 1;
    variant_counter(HLANC_KL_BASIS_FP64) += 1;
}

void launch_finalize(const Problem *P_d, int nprob, int, cudaStream_t s) {
    prof_begin(s);
    k_finalize<<<nprob, RTPB, 0, s>>>(P_d);
    prof_end(KC_AUX, s);
    launch_counter() += 1;
}

// Ritz vectors on the tensor cores (FP64-accurate digit splitting) where
// the shape fits, else on the FP64 CUDA cores.
void launch_ritz(const Problem *P_d, const Tile *tiles_d, int ntiles, int max_ncv, bool tensor_cores,
                 cudaStream_t s) {
    if (tensor_cores && ritz_tc_fits(max_ncv)) {
        launch_ritz_tc(P_d, tiles_d, ntiles, s);
        return;
    }
    const size_t smem = sizeof(double) * (size_t)max_ncv * RITZ_PANEL;
    static std::atomic<unsigned long long> attr{0};
    smem_limit_once(k_ritz, 64 * 1024, attr);
    prof_begin(s);
    k_ritz<<<ntiles, TPB, smem, s>>>(P_d, tiles_d);
    prof_end(KC_RITZ, s);
    launch_counter() += 1;
    variant_counter(HLANC_KL_RITZ_FP64) += 1;
}

}  // namespace hlanc
