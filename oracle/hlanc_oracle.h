/*
 * hlanc_oracle.h -- CPU oracle for the HLanc implicitly restarted Lanczos path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code.  It is imported by the test-suite, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg, always as the
 * checker (or as the timed CPU baseline), never as the product path.
 *
 * It is a plain-C restatement of the reference's CPU solver
 * (HLanc.hpp: ds_solver_mkl + dcsrmv_operator_mkl + dcsr_matrix_t).  The
 * LAPACK/BLAS routines the reference calls through MKL (dsteqr, dlartg,
 * dgeqr2, dorm2r, dgemv, dnrm2) are written from their published
 * mathematical definitions (Golub & Van Loan, "Matrix Computations", 4th ed.,
 * sections 5.1 and 8.3; Anderson, "Algorithm 978: Safe scaling in the Level 1
 * BLAS", ACM TOMS 2017, for the Givens convention), not from library source.
 *
 * Parity of this restatement is pinned against the reference's own
 * ds_solver_mkl compiled in the development container (oracle/build_ref.sh)
 * through the golden fixtures in tests/golden/.
 */
#ifndef HLANC_ORACLE_H
#define HLANC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Host CSR matrix, the data model of dcsr_matrix_t (HLanc.hpp:74-100). */
typedef struct {
    int nrows;        /* csr_row_ptr.size() - 1                        */
    int ncols;        /* num_columns                                    */
    int nnz;          /* csr_value.size() (may exceed row_ptr[nrows])   */
    int symmetric;    /* is_symmetric: only the lower triangle is stored */
    int *row_ptr;     /* nrows + 1                                      */
    int *col;         /* nnz                                            */
    double *val;      /* nnz                                            */
} ocsr_t;

/* Readers/writers, HLanc.hpp:103-392.  Return 0 on success, nonzero on a
 * read/parse error (the reference calls exit(1) there). */
int  ocsr_read(const char *format, const char *filename, int is_symmetric, ocsr_t *out);
int  ocsr_save_pp(const ocsr_t *m, const char *filename);
int  ocsr_save_mm(const ocsr_t *m, const char *filename);
int  ocsr_save_bin(const ocsr_t *m, const char *filename);
void ocsr_free(ocsr_t *m);
/* Build from caller arrays (copied). */
int  ocsr_from_arrays(int nrows, int ncols, int nnz, int symmetric, const int *row_ptr,
                      const int *col, const double *val, ocsr_t *out);

/* y = A x with dcsrmv_operator_naive semantics (HLanc.hpp:403-431). */
void ocsr_spmv_naive(const ocsr_t *m, const double *x, double *y);
/* y = A x with mkl_dcsrmv "GLNC"/"SLNC" semantics (HLanc.hpp:445-466):
 * symmetric matrices use only stored entries with col <= row. */
void ocsr_spmv_mkl(const ocsr_t *m, const double *x, double *y);
/* Expand a symmetric-lower matrix into general CSR (rows sorted by column is
 * not required); used for the multi-threaded baseline SpMV. */
int  ocsr_expand_general(const ocsr_t *m, ocsr_t *out);
/* y = A x over a general CSR, OpenMP-parallel over rows. */
void ocsr_spmv_general_omp(const ocsr_t *m, const double *x, double *y);

/* SpMV callback: y = A x for vectors of length n. */
typedef void (*oracle_spmv_fn)(void *ctx, const double *x, double *y);

typedef struct {
    long spmv_calls;     /* operator applications                            */
    int  restarts;       /* restart cycles run (loop iterations, H:1684)     */
    int  nconv;          /* converged Ritz values at exit                    */
    long cgs_passes;     /* CGS passes (first passes + DGKS corrections)     */
    double rnorm;        /* final residual norm                              */
    double cycle_seconds;/* wall time of the last restart cycle the loop ran  */
    long cycle_spmv;     /* its operator applications                        */
    int cycle_k;         /* its first Lanczos step (the kept columns)        */
} oracle_stats_t;

/* Optional per-cycle trace of the next solves on this thread (timing
 * calibration of the CPU baseline): for loop iteration i < cap, buf[3i..3i+2]
 * = seconds, operator applications, first Lanczos step.  buf = NULL stops. */
void oracle_set_trace(double *buf, int cap);

/* ds_solver restatement (HLanc.hpp:1650-1850) with mat_v_mkl_t storage
 * (HLanc.hpp:900-948): V lives in `vectors` (ldv >= n, ncv columns).
 *   start  : the start vector dgetv0 would produce (length n); the reference
 *            draws it from dlarnv with a fixed seed (HLanc.hpp:1369-1374).
 *   tol    : convergence tolerance; <= 0 means the reference's dlamch("E").
 *   max_iter: restart limit; <= 0 means the reference's MAX_ITER = 200.
 * Returns 0 on success and 1 on the reference's failure exits. */
int oracle_ds_solver(int n, int nev, int ncv, double *values, double *vectors, int ldv,
                     oracle_spmv_fn op, void *op_ctx, const double *start, double tol,
                     int max_iter, oracle_stats_t *stats);

/* Convenience: solve with a CSR matrix through ocsr_spmv_mkl (threads <= 1)
 * or through the expanded general OpenMP SpMV (threads > 1). */
int oracle_solve_csr(const ocsr_t *m, int nev, int ncv, double *values, double *vectors,
                     int ldv, const double *start, double tol, int max_iter, int threads,
                     oracle_stats_t *stats);

/* Symmetric tridiagonal eigensolver (implicit QR with Wilkinson shift,
 * Golub & Van Loan Alg. 8.3.2/8.3.3).  d[n] diagonal, e[n-1] sub-diagonal,
 * z (ldz x n) receives eigenvectors when want_z.  Eigenvalues ascending.
 * Returns 0 on success, 1 if it failed to converge. */
int oracle_tridiag_eig(int n, double *d, double *e, double *z, int ldz, int want_z);

/* Number of OpenMP threads used by the parallel kernels (1 when built
 * without OpenMP). */
int oracle_set_threads(int threads);

#ifdef __cplusplus
}
#endif
#endif
