/*
 * hlanc_oracle.c -- CPU oracle (test infrastructure only) for the HLanc IRLM
 * hot path.  See hlanc_oracle.h for scope and provenance.
 *
 * Every routine cites the reference lines it restates (HLanc.hpp:<line>).
 * Library routines the reference takes from MKL/LAPACK are restated from
 * their published definitions:
 *   - dgemv / dnrm2        : textbook dense matrix-vector product and 2-norm;
 *   - dlartg               : Givens generation with c >= 0 and r carrying the
 *                            sign of f (Anderson, ACM TOMS 2017, Alg. 978);
 *   - dsteqr("I")          : implicit symmetric tridiagonal QR with Wilkinson
 *                            shift, eigenvalues ascending (Golub & Van Loan,
 *                            Matrix Computations 4e, Alg. 8.3.2 / 8.3.3);
 *   - dgeqr2 / dorm2r      : Householder QR and its right application
 *                            (Golub & Van Loan 4e, Alg. 5.1.1 / 5.2.1).
 */
#include "hlanc_oracle.h"

#include <ctype.h>
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* small growable arrays                                                     */
/* ------------------------------------------------------------------------ */
typedef struct { int *p; long n, cap; } ivec_t;
typedef struct { double *p; long n, cap; } dvec_t;

static int ivec_push(ivec_t *v, int x) {
    if (v->n == v->cap) {
        long nc = v->cap ? v->cap * 2 : 64;
        int *np_ = (int *)realloc(v->p, (size_t)nc * sizeof(int));
        if (!np_) return 1;
        v->p = np_; v->cap = nc;
    }
    v->p[v->n++] = x;
    return 0;
}
static int dvec_push(dvec_t *v, double x) {
    if (v->n == v->cap) {
        long nc = v->cap ? v->cap * 2 : 64;
        double *np_ = (double *)realloc(v->p, (size_t)nc * sizeof(double));
        if (!np_) return 1;
        v->p = np_; v->cap = nc;
    }
    v->p[v->n++] = x;
    return 0;
}

void ocsr_free(ocsr_t *m) {
    if (!m) return;
    free(m->row_ptr); free(m->col); free(m->val);
    memset(m, 0, sizeof(*m));
}

static void ocsr_take(ocsr_t *out, ivec_t *rp, ivec_t *ci, dvec_t *v, int ncols, int sym) {
    out->nrows = (int)rp->n - 1;
    out->ncols = ncols;
    out->nnz = (int)v->n;
    out->symmetric = sym;
    out->row_ptr = rp->p;
    out->col = ci->p ? ci->p : (int *)malloc(sizeof(int));
    out->val = v->p ? v->p : (double *)malloc(sizeof(double));
}

int ocsr_from_arrays(int nrows, int ncols, int nnz, int symmetric, const int *row_ptr,
                     const int *col, const double *val, ocsr_t *out) {
    memset(out, 0, sizeof(*out));
    out->nrows = nrows; out->ncols = ncols; out->nnz = nnz; out->symmetric = symmetric ? 1 : 0;
    out->row_ptr = (int *)malloc((size_t)(nrows + 1) * sizeof(int));
    out->col = (int *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int));
    out->val = (double *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(double));
    if (!out->row_ptr || !out->col || !out->val) { ocsr_free(out); return 1; }
    memcpy(out->row_ptr, row_ptr, (size_t)(nrows + 1) * sizeof(int));
    if (nnz > 0) {
        memcpy(out->col, col, (size_t)nnz * sizeof(int));
        memcpy(out->val, val, (size_t)nnz * sizeof(double));
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Readers (HLanc.hpp:103-285)                                               */
/* ------------------------------------------------------------------------ */

/* read_pp, HLanc.hpp:120-169.  "col:val" tokens separated by blanks, one row
 * per '\n'; zero values are dropped; with is_symmetric, entries above the
 * diagonal are dropped.  A final row without a terminating '\n' contributes
 * its entries to col/val but no row_ptr entry (the reference behaves so). */
static int read_pp(const char *filename, int is_symmetric, ocsr_t *out) {
    FILE *fp = fopen(filename, "r");
    if (!fp) return 1;
    ivec_t rp = {0}, ci = {0};
    dvec_t vv = {0};
    int num_columns = 0;
    int err = ivec_push(&rp, 0);
    for (; !err;) {
        int ich;
        while (ich = fgetc(fp), (ich == ' ' || ich == '\t')) { }
        if (ich == '\n') { err = ivec_push(&rp, (int)vv.n); continue; }
        if (ich == EOF) break;
        ungetc(ich, fp);
        int index; double value;
        if (fscanf(fp, "%d:%lf", &index, &value) != 2) { err = 2; break; }
        if (value == 0.0) continue;
        int current_row = (int)rp.n - 1;
        if (!(is_symmetric && index > current_row)) {
            err |= ivec_push(&ci, index);
            err |= dvec_push(&vv, value);
        }
        if (num_columns < index) num_columns = index;
        if (is_symmetric && num_columns < current_row) num_columns = current_row;
    }
    ++num_columns;
    fclose(fp);
    if (err) { free(rp.p); free(ci.p); free(vv.p); return err; }
    ocsr_take(out, &rp, &ci, &vv, num_columns, is_symmetric ? 1 : 0);
    return 0;
}

/* read_mm, HLanc.hpp:172-247.  MatrixMarket coordinate; banner decides
 * symmetric/general; 1-based -> 0-based; zeros dropped; entries kept in file
 * order within a row; symmetric files keep only col <= row. */
static int read_mm(const char *filename, ocsr_t *out) {
    FILE *fp = fopen(filename, "r");
    if (!fp) return 1;
    char line[4096];
    if (!fgets(line, sizeof line, fp)) { fclose(fp); return 2; }
    if (strncmp(line, "%%MatrixMarket matrix coordinate", 32) != 0) { fclose(fp); return 3; }
    int sym;
    if (strstr(line, "symmetric")) sym = 1;
    else if (strstr(line, "general")) sym = 0;
    else { fclose(fp); return 3; }
    int ich;
    while ((ich = fgetc(fp)) == '%') {
        while ((ich = fgetc(fp)) != '\n' && ich != EOF) { }
        if (ich == EOF) break;
    }
    if (ich != EOF) ungetc(ich, fp);
    int rows, columns, entries;
    if (fscanf(fp, "%d%d%d", &rows, &columns, &entries) != 3 || rows < 0 || entries < 0) {
        fclose(fp); return 4;
    }
    /* Two passes over a buffered triplet list reproduce the per-row
     * push_back order of the reference's line_t vectors. */
    int *tr = (int *)malloc((size_t)(entries > 0 ? entries : 1) * sizeof(int));
    int *tc = (int *)malloc((size_t)(entries > 0 ? entries : 1) * sizeof(int));
    double *tv = (double *)malloc((size_t)(entries > 0 ? entries : 1) * sizeof(double));
    int *cnt = (int *)calloc((size_t)rows + 1, sizeof(int));
    if (!tr || !tc || !tv || !cnt) { fclose(fp); free(tr); free(tc); free(tv); free(cnt); return 5; }
    int kept = 0;
    for (int e = 0; e < entries; ++e) {
        int r, c; double v;
        if (fscanf(fp, "%d%d%lf", &r, &c, &v) != 3) {
            fclose(fp); free(tr); free(tc); free(tv); free(cnt); return 6;
        }
        if (v == 0.0) continue;
        --r; --c;
        if (r < 0 || r >= rows) {   /* out-of-range row: undefined in the reference */
            fclose(fp); free(tr); free(tc); free(tv); free(cnt); return 7;
        }
        if (sym && c > r) continue;   /* HLanc.hpp:236-239 */
        tr[kept] = r; tc[kept] = c; tv[kept] = v; ++kept;
        cnt[r + 1]++;
    }
    fclose(fp);
    for (int r = 0; r < rows; ++r) cnt[r + 1] += cnt[r];
    int *rp = (int *)malloc((size_t)(rows + 1) * sizeof(int));
    int *ci = (int *)malloc((size_t)(kept > 0 ? kept : 1) * sizeof(int));
    double *cv = (double *)malloc((size_t)(kept > 0 ? kept : 1) * sizeof(double));
    int *cur = (int *)malloc((size_t)(rows > 0 ? rows : 1) * sizeof(int));
    if (!rp || !ci || !cv || !cur) { free(tr); free(tc); free(tv); free(cnt); free(rp); free(ci); free(cv); free(cur); return 5; }
    memcpy(rp, cnt, (size_t)(rows + 1) * sizeof(int));
    for (int r = 0; r < rows; ++r) cur[r] = rp[r];
    for (int e = 0; e < kept; ++e) {
        int p = cur[tr[e]]++;
        ci[p] = tc[e]; cv[p] = tv[e];
    }
    free(tr); free(tc); free(tv); free(cnt); free(cur);
    out->nrows = rows; out->ncols = columns; out->nnz = kept; out->symmetric = sym;
    out->row_ptr = rp; out->col = ci; out->val = cv;
    return 0;
}

/* read_bin, HLanc.hpp:250-285: [ncols][nrows][row_ptr[nrows+1]][nnz]
 * [col[nnz]][val[nnz]], native int32/float64; always general. */
static int read_bin(const char *filename, ocsr_t *out) {
    FILE *fp = fopen(filename, "rb");
    if (!fp) return 1;
    int ncols, nrows, nnz;
    if (fread(&ncols, sizeof(int), 1, fp) != 1) { fclose(fp); return 2; }
    if (fread(&nrows, sizeof(int), 1, fp) != 1 || nrows < 0) { fclose(fp); return 2; }
    int *rp = (int *)malloc((size_t)(nrows + 1) * sizeof(int));
    if (!rp) { fclose(fp); return 5; }
    if (fread(rp, sizeof(int), (size_t)nrows + 1, fp) != (size_t)nrows + 1) { free(rp); fclose(fp); return 2; }
    if (fread(&nnz, sizeof(int), 1, fp) != 1 || nnz < 0) { free(rp); fclose(fp); return 2; }
    int *ci = (int *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int));
    double *cv = (double *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(double));
    if (!ci || !cv) { free(rp); free(ci); free(cv); fclose(fp); return 5; }
    if ((size_t)nnz != fread(ci, sizeof(int), (size_t)nnz, fp) ||
        (size_t)nnz != fread(cv, sizeof(double), (size_t)nnz, fp)) {
        free(rp); free(ci); free(cv); fclose(fp); return 2;
    }
    fclose(fp);
    out->nrows = nrows; out->ncols = ncols; out->nnz = nnz; out->symmetric = 0;
    out->row_ptr = rp; out->col = ci; out->val = cv;
    return 0;
}

int ocsr_read(const char *format, const char *filename, int is_symmetric, ocsr_t *out) {
    memset(out, 0, sizeof(*out));
    if (!strcmp(format, "pp")) return read_pp(filename, is_symmetric, out);
    if (!strcmp(format, "mm")) return read_mm(filename, out);
    if (!strcmp(format, "bin")) return read_bin(filename, out);
    return 9;
}

/* ------------------------------------------------------------------------ */
/* Writers (HLanc.hpp:287-392)                                               */
/* ------------------------------------------------------------------------ */
int ocsr_save_pp(const ocsr_t *m, const char *filename) {
    FILE *fp = fopen(filename, "w");
    if (!fp) return 1;
    for (int r = 0; r < m->nrows; ++r)
        for (int i = m->row_ptr[r]; i < m->row_ptr[r + 1]; ++i)
            if (fprintf(fp, "%d:%g%c", m->col[i], m->val[i], i + 1 == m->row_ptr[r + 1] ? '\n' : ' ') < 0) {
                fclose(fp); return 2;
            }
    fclose(fp);
    return 0;
}

int ocsr_save_mm(const ocsr_t *m, const char *filename) {
    FILE *fp = fopen(filename, "w");
    if (!fp) return 1;
    if (fprintf(fp, "%%%%MatrixMarket matrix coordinate real %s\n", m->symmetric ? "symmetric" : "general") < 0 ||
        fprintf(fp, "%d %d %d\n", m->nrows, m->ncols, m->nnz) < 0) { fclose(fp); return 2; }
    for (int r = 0; r < m->nrows; ++r)
        for (int i = m->row_ptr[r]; i < m->row_ptr[r + 1]; ++i)
            if (fprintf(fp, "%d %d %g\n", r + 1, m->col[i] + 1, m->val[i]) < 0) { fclose(fp); return 2; }
    fclose(fp);
    return 0;
}

/* save_bin, HLanc.hpp:331-392: a symmetric matrix is expanded to general
 * CSR; row r's entries are appended in the order the reference's loop visits
 * them (rows ascending, stored order within a row), own entries and mirrored
 * entries interleaved by visit time. */
int ocsr_save_bin(const ocsr_t *m, const char *filename) {
    ocsr_t g;
    int rc = ocsr_expand_general(m, &g);
    if (rc) return rc;
    FILE *fp = fopen(filename, "wb");
    if (!fp) { ocsr_free(&g); return 1; }
    int ok = fwrite(&g.ncols, sizeof(int), 1, fp) == 1 &&
             fwrite(&g.nrows, sizeof(int), 1, fp) == 1 &&
             fwrite(g.row_ptr, sizeof(int), (size_t)g.nrows + 1, fp) == (size_t)g.nrows + 1 &&
             fwrite(&g.nnz, sizeof(int), 1, fp) == 1 &&
             fwrite(g.col, sizeof(int), (size_t)g.nnz, fp) == (size_t)g.nnz &&
             fwrite(g.val, sizeof(double), (size_t)g.nnz, fp) == (size_t)g.nnz;
    fclose(fp);
    ocsr_free(&g);
    return ok ? 0 : 2;
}

int ocsr_expand_general(const ocsr_t *m, ocsr_t *out) {
    int n = m->nrows;
    memset(out, 0, sizeof(*out));
    int *cnt = (int *)calloc((size_t)n + 1, sizeof(int));
    if (!cnt) return 5;
    for (int r = 0; r < n; ++r)
        for (int i = m->row_ptr[r]; i < m->row_ptr[r + 1]; ++i) {
            int c = m->col[i];
            cnt[r + 1]++;
            if (m->symmetric && r != c) {
                if (c < 0 || c >= n) { free(cnt); return 7; }
                cnt[c + 1]++;
            }
        }
    for (int r = 0; r < n; ++r) cnt[r + 1] += cnt[r];
    int total = cnt[n];
    out->row_ptr = (int *)malloc((size_t)(n + 1) * sizeof(int));
    out->col = (int *)malloc((size_t)(total > 0 ? total : 1) * sizeof(int));
    out->val = (double *)malloc((size_t)(total > 0 ? total : 1) * sizeof(double));
    int *cur = (int *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
    if (!out->row_ptr || !out->col || !out->val || !cur) { free(cnt); free(cur); ocsr_free(out); return 5; }
    memcpy(out->row_ptr, cnt, (size_t)(n + 1) * sizeof(int));
    for (int r = 0; r < n; ++r) cur[r] = cnt[r];
    for (int r = 0; r < n; ++r)
        for (int i = m->row_ptr[r]; i < m->row_ptr[r + 1]; ++i) {
            int c = m->col[i];
            double v = m->val[i];
            int p = cur[r]++;
            out->col[p] = c; out->val[p] = v;
            if (m->symmetric && r != c) {
                int q = cur[c]++;
                out->col[q] = r; out->val[q] = v;
            }
        }
    free(cnt); free(cur);
    out->nrows = n; out->ncols = m->ncols; out->nnz = total; out->symmetric = 0;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* SpMV                                                                      */
/* ------------------------------------------------------------------------ */
void ocsr_spmv_naive(const ocsr_t *m, const double *x, double *y) {
    int n = m->nrows;
    if (m->symmetric) {   /* HLanc.hpp:408-419 */
        for (int i = 0; i < n; ++i) y[i] = 0.0;
        for (int r = 0; r < n; ++r)
            for (int i = m->row_ptr[r]; i < m->row_ptr[r + 1]; ++i) {
                int c = m->col[i];
                double v = m->val[i];
                y[r] += x[c] * v;
                if (r != c) y[c] += x[r] * v;
            }
    } else {              /* HLanc.hpp:421-429 */
        for (int r = 0; r < n; ++r) {
            double s = 0.0;
            for (int i = m->row_ptr[r]; i < m->row_ptr[r + 1]; ++i) s += x[m->col[i]] * m->val[i];
            y[r] = s;
        }
    }
}

/* mkl_dcsrmv("N", alpha=1, "SLNC" or "GLNC", beta=0), the call at
 * HLanc.hpp:452-465: for 'S' only the stored lower triangle (col <= row) is
 * used and mirrored. */
void ocsr_spmv_mkl(const ocsr_t *m, const double *x, double *y) {
    int n = m->nrows;
    if (!m->symmetric) { ocsr_spmv_naive(m, x, y); return; }
    for (int i = 0; i < n; ++i) y[i] = 0.0;
    for (int r = 0; r < n; ++r)
        for (int i = m->row_ptr[r]; i < m->row_ptr[r + 1]; ++i) {
            int c = m->col[i];
            if (c > r) continue;
            double v = m->val[i];
            y[r] += v * x[c];
            if (c < r) y[c] += v * x[r];
        }
}

void ocsr_spmv_general_omp(const ocsr_t *m, const double *x, double *y) {
    int n = m->nrows;
    const int *rp = m->row_ptr, *ci = m->col;
    const double *v = m->val;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < n; ++r) {
        double s = 0.0;
        for (int i = rp[r]; i < rp[r + 1]; ++i) s += v[i] * x[ci[i]];
        y[r] = s;
    }
}

int oracle_set_threads(int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
    return omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* dense helpers (textbook BLAS-1/2)                                         */
/* ------------------------------------------------------------------------ */
static double dnrm2(long n, const double *x) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static) if (n > 65536)
    for (long i = 0; i < n; ++i) s += x[i] * x[i];
    return sqrt(s);
}

/* Row blocks that keep a slice of x (or y) in a core's L1 while every
 * column streams past it once. */
#define ORACLE_ROW_BLOCK 2048

/* y[0:c) = V[:, 0:c)^T x   (cblas_dgemv Trans, alpha=1, beta=0) */
static void gemv_t(long n, int c, const double *v, long ldv, const double *x, double *y) {
    for (int k = 0; k < c; ++k) y[k] = 0.0;
#ifdef _OPENMP
    int nt = n > 65536 ? omp_get_max_threads() : 1;
#else
    int nt = 1;
#endif
    double *part = (double *)calloc((size_t)nt * (size_t)c, sizeof(double));
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        int t = omp_get_thread_num();
        int T = omp_get_num_threads();
#else
        int t = 0, T = 1;
#endif
        long lo = n * t / T, hi = n * (t + 1) / T;
        double *pk = part + (size_t)t * c;
        for (long b = lo; b < hi; b += ORACLE_ROW_BLOCK) {
            long e = b + ORACLE_ROW_BLOCK < hi ? b + ORACLE_ROW_BLOCK : hi;
            for (int k = 0; k < c; ++k) {
                const double *vk = v + (long)k * ldv;
                double s = 0.0;
                for (long i = b; i < e; ++i) s += vk[i] * x[i];
                pk[k] += s;
            }
        }
    }
    for (int t = 0; t < nt; ++t)
        for (int k = 0; k < c; ++k) y[k] += part[(size_t)t * c + k];
    free(part);
}

/* y = beta*y + alpha * V[:, 0:c) x   (cblas_dgemv NoTrans), column-axpy
 * form over row blocks */
static void gemv_n(long n, int c, double alpha, const double *v, long ldv, const double *x,
                   double beta, double *y) {
#pragma omp parallel for schedule(static) if (n > 65536)
    for (long b = 0; b < n; b += ORACLE_ROW_BLOCK) {
        long e = b + ORACLE_ROW_BLOCK < n ? b + ORACLE_ROW_BLOCK : n;
        double acc[ORACLE_ROW_BLOCK];
        for (long i = b; i < e; ++i) acc[i - b] = 0.0;
        for (int k = 0; k < c; ++k) {
            const double *vk = v + (long)k * ldv;
            const double xk = x[k];
            for (long i = b; i < e; ++i) acc[i - b] += vk[i] * xk;
        }
        for (long i = b; i < e; ++i) y[i] = (beta == 0.0 ? 0.0 : beta * y[i]) + alpha * acc[i - b];
    }
}

/* Givens generation with the dlartg convention of LAPACK >= 3.10 (the
 * definition in Anderson, ACM TOMS 2017): g == 0 -> (1, 0, f); f == 0 ->
 * (0, sign(g), |g|); otherwise d = sqrt(f^2+g^2), c = |f|/d, r = sign(f) d,
 * s = g/r.  Scaling guards the extreme ranges. */
static void givens(double f, double g, double *c, double *s, double *r) {
    if (g == 0.0) { *c = 1.0; *s = 0.0; *r = f; return; }
    if (f == 0.0) { *c = 0.0; *s = copysign(1.0, g); *r = fabs(g); return; }
    double f1 = fabs(f), g1 = fabs(g);
    const double rtmin = sqrt(DBL_MIN), rtmax = sqrt(DBL_MAX / 2);
    double d;
    if (f1 > rtmin && f1 < rtmax && g1 > rtmin && g1 < rtmax) {
        d = sqrt(f * f + g * g);
        *c = f1 / d;
        *r = copysign(d, f);
        *s = g / *r;
    } else {
        double u = fmin(DBL_MAX, fmax(DBL_MIN, fmax(f1, g1)));
        double fs = f / u, gs = g / u;
        d = sqrt(fs * fs + gs * gs);
        *c = fabs(fs) / d;
        *r = copysign(d, f);
        *s = gs / *r;
        *r *= u;
    }
}

/* ------------------------------------------------------------------------ */
/* symmetric tridiagonal QR (replaces dsteqr("I"), HLanc.hpp:1691/1805)      */
/* ------------------------------------------------------------------------ */
int oracle_tridiag_eig(int n, double *d, double *e, double *z, int ldz, int want_z) {
    const double eps = DBL_EPSILON * 0.5;
    if (want_z) {
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) z[i + (long)j * ldz] = (i == j) ? 1.0 : 0.0;
    }
    if (n <= 1) return 0;
    int hi = n - 1;
    long iters = 0, maxit = 30L * n;
    while (hi > 0) {
        for (int i = 0; i < hi; ++i)
            if (fabs(e[i]) <= eps * (fabs(d[i]) + fabs(d[i + 1])) || fabs(e[i]) < DBL_MIN) e[i] = 0.0;
        while (hi > 0 && e[hi - 1] == 0.0) --hi;
        if (hi == 0) break;
        int lo = hi - 1;
        while (lo > 0 && e[lo - 1] != 0.0) --lo;
        if (++iters > maxit) return 1;
        /* Wilkinson shift from the trailing 2x2 of the block (Alg. 8.3.2). */
        double dd = 0.5 * (d[hi - 1] - d[hi]);
        double b = e[hi - 1];
        double den = dd + copysign(hypot(dd, b), dd);
        double mu = (den != 0.0) ? d[hi] - b * (b / den) : d[hi] - fabs(b);
        double x = d[lo] - mu, zz = e[lo];
        for (int k = lo; k < hi; ++k) {
            double r = hypot(x, zz);
            double c = 1.0, s = 0.0;
            if (r != 0.0) { c = x / r; s = zz / r; }
            if (k > lo) e[k - 1] = r;
            double ak = d[k], ak1 = d[k + 1], bk = e[k];
            d[k] = c * c * ak + 2.0 * c * s * bk + s * s * ak1;
            d[k + 1] = s * s * ak - 2.0 * c * s * bk + c * c * ak1;
            e[k] = c * s * (ak1 - ak) + (c * c - s * s) * bk;
            if (k < hi - 1) {
                zz = s * e[k + 1];
                e[k + 1] = c * e[k + 1];
                x = e[k];
            }
            if (want_z) {
                double *zk = z + (long)k * ldz, *zk1 = z + (long)(k + 1) * ldz;
                for (int i = 0; i < n; ++i) {
                    double a0 = zk[i], a1 = zk1[i];
                    zk[i] = c * a0 + s * a1;
                    zk1[i] = -s * a0 + c * a1;
                }
            }
        }
    }
    /* ascending order, selection sort (stable for distinct values) */
    for (int i = 0; i < n - 1; ++i) {
        int k = i;
        for (int j = i + 1; j < n; ++j) if (d[j] < d[k]) k = j;
        if (k != i) {
            double t = d[i]; d[i] = d[k]; d[k] = t;
            if (want_z)
                for (int r = 0; r < n; ++r) {
                    double tz = z[r + (long)i * ldz];
                    z[r + (long)i * ldz] = z[r + (long)k * ldz];
                    z[r + (long)k * ldz] = tz;
                }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* IRLM pieces                                                               */
/* ------------------------------------------------------------------------ */
typedef struct { double d1, d2; } d2_t;   /* HLanc.hpp:1353-1358 */

/* Stable merge sort on d2_t with a comparison selector, so the oracle's
 * order is deterministic on ties (std::sort in the reference is not). */
enum { BY_D1_ASC, BY_D1_DESC, BY_D2_ASC, BY_D2_DESC };
static int d2_before(const d2_t *a, const d2_t *b, int how) {
    switch (how) {
    case BY_D1_ASC: return a->d1 < b->d1;
    case BY_D1_DESC: return a->d1 > b->d1;
    case BY_D2_ASC: return a->d2 < b->d2;
    default: return a->d2 > b->d2;
    }
}
static void d2_sort(d2_t *p, int n, int how) {
    /* insertion sort: n <= ncv (small) */
    for (int i = 1; i < n; ++i) {
        d2_t x = p[i];
        int j = i - 1;
        while (j >= 0 && d2_before(&x, &p[j], how)) { p[j + 1] = p[j]; --j; }
        p[j + 1] = x;
    }
}

/* dsconv, HLanc.hpp:1377-1384 */
static int dsconv(int n, const double *ritz, const double *bounds, double tol, double eps23) {
    int nconv = 0;
    for (int i = 0; i < n; ++i) {
        double temp = fmax(eps23, fabs(ritz[i]));
        nconv += bounds[i] <= tol * temp;
    }
    return nconv;
}

/* dsgets, HLanc.hpp:1387-1401: sort all ncv by Ritz value ascending, then the
 * first np (unwanted, used as exact shifts) by bound descending. */
static void dsgets(int nev, int np, double *ritz, double *bounds) {
    int ncv = nev + np;
    d2_t p[ncv > 0 ? ncv : 1];
    for (int i = 0; i < ncv; ++i) { p[i].d1 = ritz[i]; p[i].d2 = bounds[i]; }
    d2_sort(p, ncv, BY_D1_ASC);
    d2_sort(p, np, BY_D2_DESC);
    for (int i = 0; i < ncv; ++i) { ritz[i] = p[i].d1; bounds[i] = p[i].d2; }
}

typedef struct {
    long n; int ncv; long ldv;
    double *v;               /* basis, column-major */
    oracle_spmv_fn op; void *ctx;
    oracle_stats_t *st;
} irlm_t;

/* one CGS pass (mat_v_mkl_t::op, HLanc.hpp:910-913):
 *   irj = V[:, 0:c)^T ipj ;  resid -= V[:, 0:c) irj */
static void cgs_pass(irlm_t *s, int c, const double *ipj, double *irj, double *resid) {
    gemv_t(s->n, c, s->v, s->ldv, ipj, irj);
    gemv_n(s->n, c, -1.0, s->v, s->ldv, irj, 1.0, resid);
    if (s->st) s->st->cgs_passes++;
}

/* dsaitr, HLanc.hpp:1404-1482: Lanczos steps j = k .. k+np-1 with full
 * CGS reorthogonalisation and the DGKS correction (factor 0.717). */
static void dsaitr(irlm_t *s, int k, int np, double *resid, double *rnorm, double *h, int ldh,
                   double *ipj, double *irj) {
    const double safmin = DBL_MIN;
    long n = s->n;
    for (int j = k; j < k + np; ++j) {
        double *vj = s->v + (long)j * s->ldv;
        if (*rnorm > safmin) {                       /* STEP 2, H:1412-1419 */
            double temp1 = 1.0 / *rnorm;
            for (long i = 0; i < n; ++i) irj[i] = resid[i] * temp1;
        } else {
            memcpy(irj, resid, (size_t)n * sizeof(double));
        }
        memcpy(vj, irj, (size_t)n * sizeof(double));  /* set_column, H:1421 */
        s->op(s->ctx, irj, resid);                    /* STEP 3, H:1424 */
        if (s->st) s->st->spmv_calls++;
        memcpy(ipj, resid, (size_t)n * sizeof(double));   /* STEP 4 */
        double wnorm = dnrm2(n, resid);
        cgs_pass(s, j + 1, ipj, irj, resid);
        h[ldh + j] = irj[j];
        h[j] = (j == 0) ? 0.0 : *rnorm;
        memcpy(ipj, resid, (size_t)n * sizeof(double));
        *rnorm = dnrm2(n, resid);
        int iter = 0;                                 /* STEP 5, H:1443-1465 */
        while (*rnorm < wnorm * 0.717) {
            cgs_pass(s, j + 1, ipj, irj, resid);
            h[ldh + j] += irj[j];
            memcpy(ipj, resid, (size_t)n * sizeof(double));
            double rnorm1 = dnrm2(n, resid);
            if (rnorm1 > *rnorm * 0.717) {
                *rnorm = rnorm1;
            } else {
                *rnorm = rnorm1;
                ++iter;
                if (iter <= 1) continue;
                for (long jj = 0; jj < n; ++jj) resid[jj] = 0.0;
                *rnorm = 0.0;
            }
            break;
        }
        if (h[j] < 0.0) {                             /* H:1467-1476 (never taken: h[j] is a norm) */
            h[j] = -h[j];
            if (j < k + np - 1) {
                double *vn = s->v + (long)(j + 1) * s->ldv;
                for (long i = 0; i < n; ++i) vn[i] = -vn[i];
            } else {
                for (long i = 0; i < n; ++i) resid[i] = -resid[i];
            }
        }
    }
}

/* dsapps, HLanc.hpp:1485-1618: np implicit shifted QR steps on the
 * tridiagonal T (bulge chase with Givens rotations), accumulated in Q, then
 * V <- V Q[:, 0:nev] and the new residual. */
static void dsapps(irlm_t *s, int nev, int np, const double *shift, double *h, int ldh,
                   double *resid, double *q, double *workd) {
    const double epsmch = DBL_EPSILON * 0.5;
    int ncv = nev + np, ldq = ncv;
    long n = s->n;
    for (int j = 0; j < ncv; ++j)
        for (int i = 0; i < ncv; ++i) q[i + j * ldq] = (i == j) ? 1.0 : 0.0;
    if (np == 0) return;
    int itop = 1;
    double c = 0.0, sn = 0.0, r = 0.0;
    for (int jj = 1; jj <= np; ++jj) {
        int istart = itop;
        for (;;) {
            int iend = ncv;
            for (int i = istart; i <= ncv - 1; ++i) {
                double big = fabs(h[ldh + i - 1]) + fabs(h[ldh + i]);
                if (h[i] <= epsmch * big) { h[i] = 0.0; iend = i; break; }
            }
            if (istart < iend) {
                double f = h[istart + ldh - 1] - shift[jj - 1];
                double g = h[istart];
                givens(f, g, &c, &sn, &r);
                double a1 = c * h[istart + ldh - 1] + sn * h[istart];
                double a2 = c * h[istart] + sn * h[istart + ldh];
                double a4 = c * h[istart + ldh] - sn * h[istart];
                double a3 = c * h[istart] - sn * h[istart + ldh - 1];
                h[istart + ldh - 1] = c * a1 + sn * a2;
                h[istart + ldh] = c * a4 - sn * a3;
                h[istart] = c * a3 + sn * a4;
                int i2 = istart + jj < ncv ? istart + jj : ncv;
                for (int j = 1; j <= i2; ++j) {
                    double t = c * q[j + (istart - 1) * ldq - 1] + sn * q[j + istart * ldq - 1];
                    q[j + istart * ldq - 1] = -sn * q[j + (istart - 1) * ldq - 1] + c * q[j + istart * ldq - 1];
                    q[j + (istart - 1) * ldq - 1] = t;
                }
                for (int i = istart + 1; i <= iend - 1; ++i) {
                    f = h[i - 1];
                    g = sn * h[i];
                    h[i] = c * h[i];
                    givens(f, g, &c, &sn, &r);
                    if (r < 0.0) { r = -r; c = -c; sn = -sn; }
                    h[i - 1] = r;
                    double b1 = c * h[i + ldh - 1] + sn * h[i];
                    double b2 = c * h[i] + sn * h[i + ldh];
                    double b3 = c * h[i] - sn * h[i + ldh - 1];
                    double b4 = c * h[i + ldh] - sn * h[i];
                    h[i + ldh - 1] = c * b1 + sn * b2;
                    h[i + ldh] = c * b4 - sn * b3;
                    h[i] = c * b3 + sn * b4;
                    int i3 = i + jj < ncv ? i + jj : ncv;
                    for (int j = 1; j <= i3; ++j) {
                        double t = c * q[j + (i - 1) * ldq - 1] + sn * q[j + i * ldq - 1];
                        q[j + i * ldq - 1] = -sn * q[j + (i - 1) * ldq - 1] + c * q[j + i * ldq - 1];
                        q[j + (i - 1) * ldq - 1] = t;
                    }
                }
            }
            istart = iend + 1;
            if (h[iend - 1] < 0.0) {
                h[iend - 1] = -h[iend - 1];
                for (int i = 0; i < ncv; ++i) q[(iend - 1) * ldq + i] *= -1.0;
            }
            if (iend < ncv) continue;
            for (int i = itop; i <= ncv - 1; ++i) {
                if (h[i] > 0.0) break;
                ++itop;
            }
            break;
        }
    }
    for (int i = itop; i <= ncv - 1; ++i) {
        double big = fabs(h[i + ldh - 1]) + fabs(h[i + ldh]);
        if (h[i] <= epsmch * big) h[i] = 0.0;
    }
    /* H:1591-1614.  workd[n..2n) = V Q[:, nev]; V[:, ncv-i] = V[:, 0:ncv-i+1] Q[., nev-i];
     * move columns; resid = resid*Q[ncv-1, nev-1] + h[nev] V'[:, nev]. */
    double *wn = workd + n, *w0 = workd;
    if (h[nev] > 0) gemv_n(n, ncv, 1.0, s->v, s->ldv, q + nev * ldq, 0.0, wn);
    for (int i = 1; i <= nev; ++i) {
        gemv_n(n, ncv - i + 1, 1.0, s->v, s->ldv, q + (nev - i) * ldq, 0.0, w0);
        memcpy(s->v + (long)(ncv - i) * s->ldv, w0, (size_t)n * sizeof(double));
    }
    memmove(s->v, s->v + (long)np * s->ldv, (size_t)nev * (size_t)s->ldv * sizeof(double));
    if (h[nev] > 0.0) memcpy(s->v + (long)nev * s->ldv, wn, (size_t)n * sizeof(double));
    double qs = q[ncv + (nev - 1) * ldq - 1];
    for (long i = 0; i < n; ++i) resid[i] *= qs;
    if (h[nev] > 0.0) {
        const double *vn = s->v + (long)nev * s->ldv;
        for (long i = 0; i < n; ++i) resid[i] += h[nev] * vn[i];
    }
}

/* dsesrt, HLanc.hpp:1626-1647: sort values[0:nconv) ascending and permute
 * the matching columns of iq. */
static void dsesrt(int nconv, double *values, int ncv, double *iq, int ldq) {
    int idx[nconv > 0 ? nconv : 1];
    for (int i = 0; i < nconv; ++i) idx[i] = i;
    for (int i = 1; i < nconv; ++i) {     /* stable insertion sort of indices */
        int x = idx[i], j = i - 1;
        while (j >= 0 && values[x] < values[idx[j]]) { idx[j + 1] = idx[j]; --j; }
        idx[j + 1] = x;
    }
    double *qq = (double *)malloc(sizeof(double) * (size_t)ldq * (size_t)(nconv > 0 ? nconv : 1));
    memcpy(qq, values, sizeof(double) * (size_t)nconv);
    for (int i = 0; i < nconv; ++i) values[i] = qq[idx[i]];
    memcpy(qq, iq, sizeof(double) * (size_t)ldq * (size_t)nconv);
    for (int c = 0; c < nconv; ++c) memcpy(iq + (long)c * ldq, qq + (long)idx[c] * ldq, sizeof(double) * (size_t)ncv);
    free(qq);
}

/* Householder QR of A (m x k, lda) in place: R on and above the diagonal,
 * reflector tails below, tau[k].  H_i = I - tau_i v v^T with v_i = 1,
 * beta = -sign(alpha) ||x|| (Golub & Van Loan 4e, Alg. 5.1.1 / 5.2.1). */
static void householder_qr(int m, int k, double *a, int lda, double *tau) {
    for (int i = 0; i < k; ++i) {
        double *col = a + i + (long)i * lda;
        int len = m - i;
        double alpha = col[0];
        double xn = 0.0;
        for (int t = 1; t < len; ++t) xn = hypot(xn, col[t]);
        if (xn == 0.0) { tau[i] = 0.0; continue; }
        double beta = -copysign(hypot(alpha, xn), alpha);
        tau[i] = (beta - alpha) / beta;
        double scal = 1.0 / (alpha - beta);
        for (int t = 1; t < len; ++t) col[t] *= scal;
        col[0] = beta;
        /* apply H_i to the trailing columns from the left */
        for (int jc = i + 1; jc < k; ++jc) {
            double *cj = a + i + (long)jc * lda;
            double w = cj[0];
            for (int t = 1; t < len; ++t) w += col[t] * cj[t];
            w *= tau[i];
            cj[0] -= w;
            for (int t = 1; t < len; ++t) cj[t] -= w * col[t];
        }
    }
}

/* C (n x m, ldc) <- C * H_0 * H_1 * ... * H_{k-1}  (dorm2r "Right","N") */
static void householder_apply_right(long n, int m, int k, const double *a, int lda,
                                    const double *tau, double *cmat, long ldc) {
    for (int i = 0; i < k; ++i) {
        if (tau[i] == 0.0) continue;
        const double *vv = a + i + (long)i * lda;   /* v[0] = 1 implied */
        int len = m - i;
#pragma omp parallel for schedule(static) if (n > 65536)
        for (long r = 0; r < n; ++r) {
            double w = cmat[r + (long)i * ldc];
            for (int t = 1; t < len; ++t) w += cmat[r + (long)(i + t) * ldc] * vv[t];
            w *= tau[i];
            cmat[r + (long)i * ldc] -= w;
            for (int t = 1; t < len; ++t) cmat[r + (long)(i + t) * ldc] -= w * vv[t];
        }
    }
}

static _Thread_local double *g_trace = NULL;
static _Thread_local int g_trace_cap = 0;
void oracle_set_trace(double *buf, int cap) { g_trace = buf; g_trace_cap = buf ? cap : 0; }

/* ds_solver, HLanc.hpp:1650-1850 */
int oracle_ds_solver(int n, int nev, int ncv, double *values, double *vectors, int ldv,
                     oracle_spmv_fn op, void *op_ctx, const double *start, double tol,
                     int max_iter, oracle_stats_t *stats) {
    if (n <= 0 || nev <= 0 || ncv <= nev || ncv > n || ldv < n) return 1;
    const double eps = DBL_EPSILON * 0.5;
    if (tol <= 0.0) tol = eps;                               /* H:1651 */
    double eps23 = pow(eps, 0.66666666666666663);           /* H:1652 */
    if (max_iter <= 0) max_iter = 200;                      /* H:1682 */
    oracle_stats_t local;
    if (!stats) stats = &local;
    memset(stats, 0, sizeof(*stats));

    int np = ncv - nev, nconv = 0, nev0 = nev, np0 = np;
    double rnorm;
    double *resid = (double *)malloc(sizeof(double) * (size_t)n);
    double *workd = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    double *ipj = (double *)malloc(sizeof(double) * (size_t)n);
    double *irj = (double *)malloc(sizeof(double) * (size_t)n);
    int lworkl = ncv * (ncv + 8);
    double *workl_alloc = (double *)calloc((size_t)lworkl, sizeof(double));
    if (!resid || !workd || !ipj || !irj || !workl_alloc) {
        free(resid); free(workd); free(ipj); free(irj); free(workl_alloc); return 1;
    }
    int ret = 1;
    /* dgetv0, H:1369-1374 (start vector supplied by the caller) */
    memcpy(resid, start, sizeof(double) * (size_t)n);
    rnorm = dnrm2(n, resid);

    double *h = workl_alloc;                 /* H:1670-1676 */
    int ldh = ncv;
    double *ritz = h + ncv * 2;
    double *bounds = ritz + ncv;
    double *q = bounds + ncv;
    int ldq = ncv;
    double *workl = q + ncv * ncv;
    double *qfull = (double *)malloc(sizeof(double) * (size_t)ncv * (size_t)ncv);
    double *ework = (double *)malloc(sizeof(double) * (size_t)ncv);

    irlm_t s = { n, ncv, ldv, vectors, op, op_ctx, stats };

    dsaitr(&s, 0, nev0, resid, &rnorm, h, ldh, ipj, irj);     /* H:1680 */

    int iter;
    for (iter = 0; iter < max_iter; ++iter) {                /* H:1684-1736 */
        stats->restarts = iter + 1;
        const double t_cycle = omp_get_wtime();
        const long spmv_cycle = stats->spmv_calls;
        const int k_cycle = nev;
        dsaitr(&s, nev, np, resid, &rnorm, h, ldh, ipj, irj);
        memcpy(ritz, h + ldh, sizeof(double) * (size_t)ncv);
        memcpy(ework, h + 1, sizeof(double) * (size_t)(ncv - 1));
        if (oracle_tridiag_eig(ncv, ritz, ework, q, ldq, 1)) goto done;
        for (int i = 0; i < ncv; ++i) bounds[i] = rnorm * fabs(q[i * ncv + ncv - 1]);
        memcpy(workl + ncv, ritz, sizeof(double) * (size_t)ncv);
        memcpy(workl + ncv * 2, bounds, sizeof(double) * (size_t)ncv);
        nev = nev0; np = np0;
        dsgets(nev, np, ritz, bounds);
        memcpy(workl + np, bounds + np, sizeof(double) * (size_t)nev);
        nconv = dsconv(nev, ritz + np, workl + np, tol, eps23);
        for (int j = 0; j < np; ++j)
            if (bounds[j] == 0.0) { --np; ++nev; }
        if (nconv >= nev0 || np == 0) break;
        int nevbef = nev;
        nev += (nconv < np / 2) ? nconv : np / 2;
        if (nev == 1 && ncv >= 6) nev = ncv / 2;
        else if (nev == 1 && ncv > 2) nev = 2;
        np = ncv - nev;
        if (nevbef < nev) dsgets(nev, np, ritz, bounds);
        dsapps(&s, nev, np, ritz, h, ldh, resid, qfull, workd);
        rnorm = dnrm2(n, resid);
        stats->cycle_seconds = omp_get_wtime() - t_cycle;     /* timing only, no effect on results */
        stats->cycle_spmv = stats->spmv_calls - spmv_cycle;
        stats->cycle_k = k_cycle;
        if (iter < g_trace_cap) {
            g_trace[3 * iter] = stats->cycle_seconds;
            g_trace[3 * iter + 1] = (double)stats->cycle_spmv;
            g_trace[3 * iter + 2] = (double)k_cycle;
        }
    }
    stats->nconv = nconv;
    stats->rnorm = rnorm;

    /* final sort of ritz/bounds, H:1738-1758 (no observable output) */
    {
        d2_t p[ncv];
        for (int i = 0; i < ncv; ++i) { p[i].d1 = ritz[i]; p[i].d2 = bounds[i]; }
        d2_sort(p, ncv, BY_D1_DESC);
        for (int j = 0; j < nev0; ++j) p[j].d2 /= fmax(eps23, fabs(p[j].d1));
        d2_sort(p, nev0, BY_D2_ASC);
        for (int j = 0; j < nev0; ++j) p[j].d2 *= fmax(eps23, fabs(p[j].d1));
        d2_sort(p, nconv, BY_D1_ASC);
        for (int i = 0; i < ncv; ++i) { ritz[i] = p[i].d1; bounds[i] = p[i].d2; }
    }
    h[0] = rnorm;
    if (nconv < nev0) goto done;

    /* eigenvectors, H:1765-1843 */
    nev = nev0; np = np0;
    {
        char select[ncv];
        for (int j = 0; j < ncv; ++j) { bounds[j] = j + 1; select[j] = 0; }
        int irz = 5 * ncv + ncv * ncv, ibd = irz + ncv;
        dsgets(nev, np, workl_alloc + irz, bounds);
        int reord = 0, numcnv = 0;
        for (int j = 0; j < ncv; ++j) {
            double temp1 = fmax(eps23, fabs(workl_alloc[irz + ncv - j - 1]));
            int jj = (int)bounds[ncv - j - 1];
            if (numcnv < nconv && workl_alloc[ibd + jj - 1] <= tol * temp1) {
                select[jj - 1] = 1;
                ++numcnv;
                if (jj > nev) reord = 1;
            }
        }
        if (numcnv != nconv) goto done;
        double *ihd = workl_alloc + ncv * 4;
        double *ihb = workl_alloc + ncv * 5;
        memcpy(ihb, h + 1, sizeof(double) * (size_t)(ncv - 1));
        memcpy(ihd, h + ldh, sizeof(double) * (size_t)ncv);
        double *iq = workl_alloc + ncv * 6;
        double *iw = iq + ncv * ncv;
        if (oracle_tridiag_eig(ncv, ihd, ihb, iq, ldq, 1)) goto done;
        if (reord) {
            int left = 0, right = ncv - 1;
            for (;;) {
                while (left < ncv && select[left]) ++left;
                while (right >= 0 && !select[right]) --right;
                if (left > right) break;
                double t = ihd[left]; ihd[left] = ihd[right]; ihd[right] = t;
                for (int i = 0; i < ncv; ++i) {
                    double tq = iq[ldq * left + i];
                    iq[ldq * left + i] = iq[ldq * right + i];
                    iq[ldq * right + i] = tq;
                }
                ++left; --right;
            }
        }
        memcpy(values, ihd, sizeof(double) * (size_t)nconv);
        dsesrt(nconv, values, ncv, iq, ldq);
        householder_qr(ncv, nconv, iq, ldq, iw);
        householder_apply_right(n, ncv, nconv, iq, ldq, iw, vectors, ldv);
    }
    ret = 0;
done:
    free(resid); free(workd); free(ipj); free(irj); free(workl_alloc); free(qfull); free(ework);
    return ret;
}

/* ------------------------------------------------------------------------ */
typedef struct { const ocsr_t *m; int general; } csr_ctx_t;
static void csr_op_mkl(void *ctx, const double *x, double *y) {
    csr_ctx_t *c = (csr_ctx_t *)ctx;
    if (c->general) ocsr_spmv_general_omp(c->m, x, y);
    else ocsr_spmv_mkl(c->m, x, y);
}

int oracle_solve_csr(const ocsr_t *m, int nev, int ncv, double *values, double *vectors,
                     int ldv, const double *start, double tol, int max_iter, int threads,
                     oracle_stats_t *stats) {
    ocsr_t g;
    csr_ctx_t ctx;
    int use_general = threads > 1;
    int saved = oracle_set_threads(0);
    oracle_set_threads(threads > 0 ? threads : 1);
    if (use_general) {
        if (m->symmetric) {
            if (ocsr_expand_general(m, &g)) { oracle_set_threads(saved); return 1; }
        } else {
            g = *m;
        }
        ctx.m = &g; ctx.general = 1;
    } else {
        ctx.m = m; ctx.general = 0;
    }
    int rc = oracle_ds_solver(m->nrows, nev, ncv, values, vectors, ldv, csr_op_mkl, &ctx, start,
                              tol, max_iter, stats);
    if (use_general && m->symmetric) ocsr_free(&g);
    oracle_set_threads(saved);
    return rc;
}
