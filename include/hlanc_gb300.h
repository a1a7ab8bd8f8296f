/*
 * hlanc_gb300.h -- C ABI of the GB300 (sm_103a) implicitly restarted Lanczos
 * library.  Plain pointers, sizes and status codes; no C++ or torch types.
 *
 * The C++ drop-in header HLanc.hpp (same directory) sits on these entry
 * points and keeps the reference's header-only API (namespace HLanc:
 * dcsr_matrix_t, dcsrmv_operator_gpu, ds_solver_gpu).  Each declaration names
 * the reference interface it replaces as HLanc.hpp:<line> of the reference
 * header (butterfly0923/HLanc).
 *
 * Every entry point returns an int status (HLANC_OK == 0).  None of them
 * exits or aborts the process; device-side waits are bounded and report
 * HLANC_ERR_DEVICE_TIMEOUT instead of hanging.
 */
#ifndef HLANC_GB300_H
#define HLANC_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define HLANC_OK                  0
#define HLANC_NOT_CONVERGED       1  /* the reference's "return 1" (HLanc.hpp:1692,1762,1792,1806,1838,1841) */
#define HLANC_ERR_INVALID         2  /* bad argument (ncv <= nev, ncv > n, ldv < n, ...) */
#define HLANC_ERR_CUDA            3  /* a CUDA runtime call failed */
#define HLANC_ERR_ALLOC           4  /* device or host allocation failed / over budget */
#define HLANC_ERR_DEVICE_TIMEOUT  5  /* a bounded device-side wait expired */
#define HLANC_ERR_IO              6  /* file open/parse/write error (matrix or eigenpair files) */
#define HLANC_ERR_UNSUPPORTED     7  /* size outside the supported envelope */
#define HLANC_ERR_CALLBACK        8  /* a host operator callback reported failure */
#define HLANC_ERR_CANCELLED       9  /* a serving request was cancelled */

/* ---- precision modes --------------------------------------------------- */
#define HLANC_PREC_FP64           0  /* FP64 SpMV (the reference's arithmetic) */
#define HLANC_PREC_FP32_REFINE    1  /* FP32 SpMV, FP64 everywhere else, FP64 refinement: a
                                        Rayleigh-Ritz of the FP32 phase's pairs with the FP64
                                        operator, accepted when every FP64 residual meets tol,
                                        else FP64 restart cycles from the refined vectors */

/* Kernel of the restart's basis update V <- V Q and of the final Ritz
 * vectors V Q2 (hlanc_opts_t.basis_kernel). */
#define HLANC_BASIS_AUTO          0  /* tensor cores (FP64-accurate integer splitting) when
                                        ncv <= 64 (so nev <= 63), else the FP64 kernels */
#define HLANC_BASIS_FP64          1  /* always the FP64 CUDA-core kernels */

/* Arithmetic of the CGS passes h = V^T w, w -= V h (hlanc_opts_t.cgs_kernel).
 * The hybrid projection runs 5 of every 8 columns as FP64 FMAs and 3 as
 * exact fixed-point integer products (inputs quantised to 2^-58 of their
 * scale, sums exact), so the FP64 and the integer pipes work at the same
 * time.  The update w -= V h reads an FP32 copy of the basis for every
 * column whose coefficient is at most 2^-32 ||w|| / c (FP32 products of
 * such terms stay within the FP64 rounding of the update) and FP64 for the
 * rest -- in a Lanczos step usually just v_j and v_{j-1}. */
#define HLANC_CGS_AUTO            0  /* hybrid projection for launches over >= 2^18 rows, else FP64;
                                        update with the FP32 copy for small coefficients */
#define HLANC_CGS_FP64            1  /* every column of both passes as FP64 FMAs */
#define HLANC_CGS_HYBRID          2  /* hybrid projection at every size; update as AUTO */

/* How a restart cycle's Lanczos steps are launched (hlanc_opts_t.cycle_kernel).
 * A problem too small to fill the GPU is latency-bound when every step is
 * seven launches; one cooperative launch can run the whole extension, its
 * CTAs meeting at bounded group barriers between the phases of a step. */
#define HLANC_CYCLE_AUTO          0  /* one launch per extension when every problem of the launch has
                                        rows of <= 96 entries and they have <= 49,152 rows in total */
#define HLANC_CYCLE_OFF           1  /* always the per-phase launches */

/* Largest ncv the device restart kernels accept, and largest nev. */
#define HLANC_MAX_NCV           128
#define HLANC_MAX_NEV            63

const char *hlanc_status_string(int status);
int hlanc_version(int *major, int *minor);   /* HLANC_VERSION_MAJOR/MINOR, HLanc.hpp:15-16 */

/* ---- host CSR matrices (dcsr_matrix_t, HLanc.hpp:74-392) ---------------- */
typedef struct hlanc_matrix_s *hlanc_matrix_t;

/* dcsr_matrix_t(format, filename, is_symmetric), HLanc.hpp:103-113:
 * format "pp" | "mm" | "bin"; parse errors return HLANC_ERR_IO. */
int hlanc_matrix_read(const char *format, const char *filename, int is_symmetric,
                      hlanc_matrix_t *out);
/* In-memory construction (copies the arrays). */
int hlanc_matrix_create(int nrows, int ncols, int nnz, const int *row_ptr, const int *col,
                        const double *val, int is_symmetric, hlanc_matrix_t *out);
/* get_num_rows/get_num_columns/get_nnz/symmetric, HLanc.hpp:83-89 */
int hlanc_matrix_info(hlanc_matrix_t m, int *nrows, int *ncols, int *nnz, int *is_symmetric);
/* get_row_ptr/get_column_index/get_value, HLanc.hpp:86-88 (borrowed pointers) */
int hlanc_matrix_arrays(hlanc_matrix_t m, const int **row_ptr, const int **col,
                        const double **val);
/* save_pp/save_mm/save_bin, HLanc.hpp:287-392 */
int hlanc_matrix_save(hlanc_matrix_t m, const char *format, const char *filename);
int hlanc_matrix_destroy(hlanc_matrix_t m);

/* ---- device CSR operator (dcsrmv_operator_gpu, HLanc.hpp:476-572) ----- */
typedef struct hlanc_csr_s *hlanc_csr_t;

/* dcsrmv_operator_gpu(m, dev), HLanc.hpp:494-514: copies the CSR to device
 * `dev` once.  A symmetric (lower-stored) matrix is expanded to general CSR
 * (cuSPARSE SYMMETRIC semantics, HLanc.hpp:512).  precision selects FP64
 * values, or FP32 values for HLANC_PREC_FP32_REFINE (the FP64 copy is kept
 * too, for refinement and residuals). */
int hlanc_csr_create(int dev, int nrows, int ncols, int nnz, const int *row_ptr, const int *col,
                     const double *val, int is_symmetric, int precision, hlanc_csr_t *out);
int hlanc_csr_destroy(hlanc_csr_t op);
int hlanc_csr_info(hlanc_csr_t op, int *dev, int *nrows, int *ncols, long long *nnz_general,
                   int *precision);
/* operator()(x, y), HLanc.hpp:531-572: y = A x; x and y may be host or
 * device pointers (device pointers on the operator's device are used in
 * place, anything else is staged).  Synchronous, like the reference. */
int hlanc_csr_apply(hlanc_csr_t op, const double *x, double *y);
/* y = A x on device pointers, asynchronous on `stream` (cudaStream_t). */
int hlanc_csr_spmv_async(hlanc_csr_t op, const double *x_d, double *y_d, void *stream);
/* FP32 SpMV (values rounded to FP32, FP32 accumulation per row). */
int hlanc_csr_spmv_f32_async(hlanc_csr_t op, const float *x_d, float *y_d, void *stream);
/* The SpMV work units hlanc_csr_create picked for this matrix (no reference
 * counterpart).  A matrix of >= 2^16 rows with rows longer than 12 entries
 * is tuned on the device: a few unit shapes (rows per unit, mean row lengths
 * at which a unit takes 4 / 8 lanes per row) and a sliced-ELL copy of the
 * matrix (rows sorted by length inside windows of 1024 rows, 32 rows per
 * warp; *rows_per_unit = -1 when it was kept) are timed and the fastest is
 * kept; us_default / us_chosen are the measured SpMV times (0 when the row
 * histogram left nothing to choose). */
int hlanc_csr_tuning(hlanc_csr_t op, int *rows_per_unit, int *lanes4_mean, int *lanes8_mean, double *us_default,
                     double *us_chosen);

/* ---- solver (ds_solver_gpu, HLanc.hpp:1868-1872 / ds_solver, 1650-1850) - */
/* Host operator callback: y = A x for host vectors of length n; return 0 on
 * success.  This is the path for any functor that is not a device CSR
 * operator (e.g. the reference demo's plain function, demo/HLanc_demo.cu:9-18). */
typedef int (*hlanc_host_op_fn)(void *ctx, const double *x, double *y);

typedef struct {
    double tol;               /* <= 0: dlamch("E"), the reference's fixed tolerance (HLanc.hpp:1651) */
    int max_restarts;         /* <= 0: 200, the reference's MAX_ITER (HLanc.hpp:1682) */
    int precision;            /* HLANC_PREC_* (must match the operator for FP32) */
    unsigned long long seed;  /* start-vector seed (SplitMix64 stream 0); default 0 */
    const double *start;      /* optional host start vector of length n (overrides seed) */
    void *stream;             /* cudaStream_t to run on; NULL = library-owned stream */
    int use_graphs;           /* replay identical restart cycles as CUDA graphs */
    int restart_on_device;    /* run the O(ncv^2) restart math in a device kernel instead of on the host */
    int profile;              /* time every kernel launch with CUDA events (eager launches); see hlanc_last_profile */
    int basis_kernel;         /* HLANC_BASIS_*; default HLANC_BASIS_AUTO */
    int cgs_kernel;           /* HLANC_CGS_*; default HLANC_CGS_AUTO */
    int wait_limit;           /* polls of each bounded device wait before it gives up and the
                                 solve returns HLANC_ERR_DEVICE_TIMEOUT: 0 = default (2^20),
                                 < 0 = give up at once (tests of the failure path) */
    int cycle_kernel;         /* HLANC_CYCLE_*; default HLANC_CYCLE_AUTO */
    int reserved[1];
} hlanc_opts_t;

/* Fill defaults (tol 0, max_restarts 200, FP64, seed 0, graphs on, host restart). */
void hlanc_opts_default(hlanc_opts_t *opts);

typedef struct {
    long long spmv_calls;     /* operator applications */
    long long cgs_passes;     /* CGS passes incl. DGKS corrections */
    int restarts;             /* restart cycles */
    int nconv;                /* converged Ritz pairs */
    int refine_restarts;      /* FP64 restart cycles after an FP32 phase */
    int status;               /* same as the return value */
    double rnorm;             /* final residual norm */
    double seconds;           /* wall time of the solve */
    double bytes_spmv;        /* algorithmic bytes moved, SpMV */
    double bytes_cgs;         /* algorithmic bytes moved, CGS passes */
    double bytes_restart;     /* algorithmic bytes moved, basis updates + Ritz vectors */
    double cgs_update_fp32_share;  /* share of the CGS update's columns read from the FP32 copy */
    double refine_residual;   /* mixed precision: largest ||A y - theta y|| / ||A||_inf after the
                                 FP64 Rayleigh-Ritz of the FP32 phase's pairs (-1: not run); the
                                 pairs were accepted as they are when refine_restarts == 0 */
    double copy_out_seconds;  /* host outputs: wall time of the device-to-host copy of the pairs */
    double reserved[1];
} hlanc_stats_t;

/* ds_solver_gpu(n, nev, ncv, values, vectors, ldv, op, dev): largest
 * algebraic eigenvalues.  values (>= ncv doubles) receives the nconv
 * converged eigenvalues ascending; vectors (host, column-major, ldv >= n,
 * ncv columns) receives the Ritz vectors in its first nconv columns and the
 * rest of the rotated basis after them, as the reference writes them.
 * Exactly one of csr / host_op is used (csr takes precedence).
 * Returns HLANC_OK, HLANC_NOT_CONVERGED (the reference's 1) or an error. */
int hlanc_solve(int dev, int n, int nev, int ncv, double *values, double *vectors, int ldv,
                hlanc_csr_t csr, hlanc_host_op_fn host_op, void *host_ctx,
                const hlanc_opts_t *opts, hlanc_stats_t *stats);

/* Same solve with device-resident outputs: values_d (ncv doubles) and
 * vectors_d (ldv_d x ncv) are device pointers on `dev`.  Used when inputs and
 * outputs stay in HBM. */
int hlanc_solve_device(int dev, int n, int nev, int ncv, double *values_d, double *vectors_d,
                       int ldv_d, hlanc_csr_t csr, const hlanc_opts_t *opts,
                       hlanc_stats_t *stats);

/* ---- residual verifier (demo/verify_eigs.cu:52-98) ---------------------- */
/* For k pairs (values[i], vectors[:, i]) on the device, computes
 * resid[i] = ||A v_i - lambda_i v_i||_2 and rdiff[i] = max_r |(Av)_r - (lambda v)_r| /
 * max(max|Av|, max|lambda v|) (verify_eigs' rdiff).  Device pointers; synchronous. */
int hlanc_residuals_device(hlanc_csr_t csr, int k, const double *values_d,
                           const double *vectors_d, int ldv_d, double *resid_h, double *rdiff_h);

/* Variant of hlanc_residuals_device that allocates nothing; it has no
 * counterpart in the reference.  For callers that cannot allocate device
 * memory when they verify Ritz pairs (a process whose HBM pool is already
 * fully claimed by its own allocator, or a loop that must not wait on a
 * cudaMalloc/cudaFree).  Its scratch is a fixed __device__ array of about
 * 513 KB, held by every GPU that loads the library until exit; k may be at
 * most HLANC_NOALLOC_MAX_PAIRS (larger k returns HLANC_ERR_UNSUPPORTED).
 * resid_h / rdiff_h are host arrays of k doubles; either may be NULL, as in
 * hlanc_residuals_device.  All calls share the scratch, so calls that
 * overlap on the GPU race; serialise them.  The first call on a device, and
 * the first after its context was re-created (cudaDeviceReset), looks up the
 * scratch address, so make those outside any stream capture.  Synchronous. */
#define HLANC_NOALLOC_MAX_PAIRS 64
int hlanc_residuals_device_noalloc(hlanc_csr_t csr, int k, const double *values_d,
                                   const double *vectors_d, int ldv_d, double *resid_h,
                                   double *rdiff_h);

/* Same check for pairs in host memory (values[k], vectors ldv x k):
 * verify_eigs' per-vector r-diff (demo/verify_eigs.cu:52-98) and ||A v - lambda v||. */
int hlanc_residuals_host(hlanc_csr_t csr, int k, const double *values_h, const double *vectors_h, int ldv_h,
                         double *resid_h, double *rdiff_h);

/* ---- eigenpair text files (demo/HLanc_solver_gpu.cu:57-66, demo/verify_eigs.cu:8-44)
 * nev, n, then nev eigenvalues and n rows of nev vector entries, "%23.15lE". */
int hlanc_eigs_write(const char *filename, int nev, int n, const double *values, const double *vectors,
                     int ldv);
/* Sizes of a file (to allocate for hlanc_eigs_read). */
int hlanc_eigs_info(const char *filename, int *nev, int *n);
/* values[nev]; vectors ldv x nev (ldv >= n), column-major. */
int hlanc_eigs_read(const char *filename, double *values, double *vectors, int ldv);

/* ---- batched solves (one launch sequence over many problems) ----------- */
typedef struct hlanc_batch_s *hlanc_batch_t;

int hlanc_batch_create(int dev, int nprob, const hlanc_csr_t *ops, const int *nev,
                       const int *ncv, const hlanc_opts_t *opts, hlanc_batch_t *out);
/* Runs every problem to completion.  values_d[i] / vectors_d[i] are device
 * outputs (ncv[i] doubles, n_i x ncv[i] with ld n_i); status[i] per problem. */
int hlanc_batch_run(hlanc_batch_t b, double **values_d, double **vectors_d, int *status,
                    hlanc_stats_t *stats);
int hlanc_batch_destroy(hlanc_batch_t b);

/* ---- serving: continuous batching of solves ----------------------------- */
typedef struct hlanc_server_s *hlanc_server_t;

typedef struct {
    size_t mem_budget_bytes;  /* admission budget: basis + workspace + Ritz output */
    int max_slots;            /* problems resident at once */
    int dev;
    int lanes;                /* launch lanes (streams) the residents are spread over;
                                 0 = 2.  A step finishes one lane's restart cycle on the
                                 host while the other lanes' cycles run on the device. */
} hlanc_server_opts_t;

/* Scheduler counters since creation (times in milliseconds). */
typedef struct {
    long long steps;          /* hlanc_server_step calls */
    long long cycles;         /* lane restart cycles completed */
    long long admitted, retired;
    double wall_ms;           /* inside hlanc_server_step */
    double wait_ms;           /* host blocked on a lane's cycle */
    double host_ms;           /* restart decisions, finalisation, result copies */
    double launch_ms;         /* enqueueing device work */
    double admin_ms;          /* admission, launch tables */
    double gpu_ms;            /* device spans of the lane cycles (overlapping lanes add up) */
    double reserved[6];
} hlanc_server_stats_t;

int hlanc_server_create(const hlanc_server_opts_t *opts, hlanc_server_t *out);
/* Submit a solve on an existing device operator; returns a request id. */
int hlanc_server_submit(hlanc_server_t s, hlanc_csr_t csr, int nev, int ncv,
                        const hlanc_opts_t *opts, long long *request_id);
/* Advance the scheduler by one restart-cycle tick (admits, runs, retires). */
int hlanc_server_step(hlanc_server_t s, int *active, int *pending);
/* Poll a request: *done = 1 when finished; then values (ncv) / vectors (n x ncv,
 * ld n, host) are filled and *status is its solve status. */
int hlanc_server_poll(hlanc_server_t s, long long request_id, int *done, int *status,
                      double *values, double *vectors, hlanc_stats_t *stats);
int hlanc_server_cancel(hlanc_server_t s, long long request_id);
int hlanc_server_stats(hlanc_server_t s, hlanc_server_stats_t *out);
int hlanc_server_destroy(hlanc_server_t s);

/* ---- diagnostics ---------------------------------------------------------- */
/* Number of kernels this library launched since load (all devices); every
 * kernel of a replayed CUDA graph counts, as if launched one by one. */
long long hlanc_kernel_launches(void);

/* Launches since load of one kernel variant (no reference counterpart; tests
 * use it to check which arithmetic a default solve took). */
#define HLANC_KL_ALL              0  /* every kernel (same as hlanc_kernel_launches) */
#define HLANC_KL_PROJ_HYBRID      1  /* CGS projection, FP64 + fixed-point panels */
#define HLANC_KL_PROJ_FP64        2  /* CGS projection, all FP64 */
#define HLANC_KL_APPLY_SHADOW     3  /* CGS update, FP32 copy for small coefficients */
#define HLANC_KL_APPLY_FP64       4  /* CGS update, all FP64 */
#define HLANC_KL_BASIS_TC         5  /* restart basis update on the tensor cores */
#define HLANC_KL_BASIS_FP64       6  /* restart basis update on FP64 CUDA cores */
#define HLANC_KL_CYCLE            7  /* a whole Lanczos extension in one cooperative launch */
#define HLANC_KL_RITZ_TC          8  /* Ritz vectors V Q2 on the tensor cores */
#define HLANC_KL_RITZ_FP64        9  /* Ritz vectors V Q2 on FP64 CUDA cores */
#define HLANC_KL_KINDS           10
long long hlanc_kernel_launches_of(int kind);

/* Per-kernel-class timing of the last solve run with opts.profile = 1 on the
 * calling thread.  Classes: 0 SpMV, 1 CGS projection, 2 CGS update,
 * 3 basis update (V*Q), 4 Ritz vectors, 5 auxiliary kernels, 6 host restart
 * (CPU time), 7 whole extensions in one launch (HLANC_CYCLE_AUTO on small
 * problems; their SpMV and CGS bytes are counted here, not in 0-2).
 * bytes / flops are the algorithmic DRAM bytes and FP64 flops of the
 * launches that did work. */
#define HLANC_PROF_CLASSES 8
typedef struct {
    long long launches[HLANC_PROF_CLASSES];
    double ms[HLANC_PROF_CLASSES];
    double bytes[HLANC_PROF_CLASSES];
    double flops[HLANC_PROF_CLASSES];
} hlanc_profile_t;
int hlanc_last_profile(hlanc_profile_t *out);

/* Measured dense FP64 FMA throughput of device `dev` (TFLOP/s): the ceiling
 * of kernels that issue one FP64 FMA per loaded 8-byte element (the
 * all-FP64 CGS kernels). */
int hlanc_diag_fp64_tflops(int dev, double *tflops);
/* The CGS kernels alone on a synthetic basis of n rows and c columns
 * (cgs_kernel HLANC_CGS_FP64 or HLANC_CGS_HYBRID), each launched reps times
 * back to back: ms3 = mean ms of a first-pass projection (with ||w||),
 * a second-pass projection and a second-pass update (its coefficients at
 * 1e-13 ||w||, so with HLANC_CGS_HYBRID every column reads the FP32 copy). */
int hlanc_diag_cgs(int dev, int n, int c, int cgs_kernel, int reps, double *ms3);

#ifdef __cplusplus
}
#endif
#endif
