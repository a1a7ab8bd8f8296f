// restart_host.h -- host-side restart and Ritz-pair selection (see restart_host.cu).
#pragma once

namespace hlanc {
namespace host {

enum { RS_APPLY = 0, RS_CONVERGED = 1, RS_NOT_CONVERGED = 2, RS_FAILED = 3 };

struct RestartIO {
    // in
    int ncv, nev0, np0, max_iter;
    double tol, eps23, rnorm;
    // in/out
    int iter;        // restart cycles completed
    double *h;       // 2*ncv: h[j] = beta_j, h[ncv + j] = alpha_j (updated by the shifts)
    // out
    double *ritz_s, *bnds_s;   // Ritz values / bounds of this cycle (ascending)
    double *Q;                 // ncv x ncv accumulated rotations (when RS_APPLY)
    int nev, np, nconv, status;
};

// One restart decision (HLanc.hpp:1686-1732): Ritz values, bounds,
// convergence test, nev/np adjustment and the implicit shifts.
int restart(RestartIO &io);

struct FinalizeIO {
    int ncv, nev0, np0, nconv;
    double tol, eps23;
    const double *h, *ritz_s, *bnds_s;
    double *values;   // out: nconv converged eigenvalues, ascending
    double *Q2;       // out: ncv x ncv orthogonal factor; Ritz vectors = V Q2
};

// Selection, reordering and Householder factor of the converged pairs
// (HLanc.hpp:1765-1842).  0 on success, 1 on the reference's failure exits.
int finalize(FinalizeIO &io);

// Symmetric tridiagonal eigensolver (implicit QR, Wilkinson shift).
int tridiag_eig(int n, double *d, double *e, double *zl, double *Z, int ldz);

// Dense symmetric eigensolver (cyclic Jacobi): A (n x n, column-major) is
// destroyed; w receives the eigenvalues ascending, Z (n x n) the
// eigenvectors as columns.  0 on success, 1 if the sweeps did not converge.
int sym_eig_jacobi(int n, double *A, double *w, double *Z);

}  // namespace host
}  // namespace hlanc
