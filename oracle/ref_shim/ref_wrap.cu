/*
 * C wrapper around the reference's unmodified CPU path (HLanc.hpp:
 * dcsr_matrix_t, dcsrmv_operator_mkl, ds_solver_mkl).  Compiled by
 * oracle/build_ref.sh into oracle/_ref/libhlanc_ref.so, a checker used only
 * in the development container to pin the oracle and to write the golden
 * fixtures under tests/golden/.  Test infrastructure, never product code.
 */
#include <HLanc.hpp>

#include <cstdio>
#include <string>
#include <unistd.h>

const double *hlanc_ref_start_vector = nullptr;

namespace {

/* dcsr_matrix_t only has file constructors (HLanc.hpp:76); a derived class
 * may fill the protected arrays after constructing from a 1x1 bin file. */
struct arrays_matrix : HLanc::dcsr_matrix_t {
    arrays_matrix(const char *dummy, int nrows, int ncols, int nnz, int sym, const int *rp,
                  const int *ci, const double *v)
        : HLanc::dcsr_matrix_t("bin", dummy) {
        csr_row_ptr.assign(rp, rp + nrows + 1);
        csr_column_index.assign(ci, ci + nnz);
        csr_value.assign(v, v + nnz);
        num_columns = ncols;
        is_symmetric = sym != 0;
    }
};

std::string dummy_bin() {
    static std::string path;
    if (path.empty()) {
        char buf[64];
        snprintf(buf, sizeof buf, "/tmp/hlanc_ref_dummy_%d.bin", (int)getpid());
        FILE *fp = fopen(buf, "wb");
        int one = 1, rp[2] = {0, 1}, c = 0;
        double v = 1.0;
        fwrite(&one, sizeof(int), 1, fp);
        fwrite(&one, sizeof(int), 1, fp);
        fwrite(rp, sizeof(int), 2, fp);
        fwrite(&one, sizeof(int), 1, fp);
        fwrite(&c, sizeof(int), 1, fp);
        fwrite(&v, sizeof(double), 1, fp);
        fclose(fp);
        path = buf;
    }
    return path;
}

template <typename op_t> struct counting_op {
    counting_op(op_t const &op) : op(op), calls(0) {}
    void operator()(double const *x, double *y) const { ++calls; op(x, y); }
    op_t const &op;
    mutable long calls;
};

HLanc::dcsr_matrix_t *g_last = nullptr;

} // namespace

extern "C" {

/* ds_solver_mkl on an in-memory CSR through dcsrmv_operator_mkl. */
int ref_solve_csr(int nrows, int ncols, int nnz, int sym, const int *rp, const int *ci,
                  const double *v, int nev, int ncv, const double *start, double *values,
                  double *vectors, int ldv, long *spmv_calls) {
    arrays_matrix m(dummy_bin().c_str(), nrows, ncols, nnz, sym, rp, ci, v);
    HLanc::dcsrmv_operator_mkl op(m);
    counting_op<HLanc::dcsrmv_operator_mkl> cop(op);
    hlanc_ref_start_vector = start;
    int rc = HLanc::ds_solver_mkl(nrows, nev, ncv, values, vectors, ldv, cop);
    hlanc_ref_start_vector = nullptr;
    if (spmv_calls) *spmv_calls = cop.calls;
    return rc;
}

/* y = A x through dcsrmv_operator_mkl and dcsrmv_operator_naive. */
void ref_spmv_csr(int nrows, int ncols, int nnz, int sym, const int *rp, const int *ci,
                  const double *v, const double *x, double *y, int naive) {
    arrays_matrix m(dummy_bin().c_str(), nrows, ncols, nnz, sym, rp, ci, v);
    if (naive) {
        HLanc::dcsrmv_operator_naive op(m);
        op(x, y);
    } else {
        HLanc::dcsrmv_operator_mkl op(m);
        op(x, y);
    }
}

/* Read a matrix with the reference reader; sizes are returned and the arrays
 * are fetched with ref_read_copy.  (The reference exits on a parse error.) */
int ref_read(const char *fmt, const char *fn, int sym, int *nrows, int *ncols, int *nnz,
             int *symflag) {
    delete g_last;
    g_last = new HLanc::dcsr_matrix_t(fmt, fn, sym != 0);
    *nrows = g_last->get_num_rows();
    *ncols = g_last->get_num_columns();
    *nnz = g_last->get_nnz();
    *symflag = g_last->symmetric() ? 1 : 0;
    return 0;
}

void ref_read_copy(int *rp, int *ci, double *v) {
    int n = g_last->get_num_rows(), z = g_last->get_nnz();
    std::memcpy(rp, g_last->get_row_ptr(), sizeof(int) * (size_t)(n + 1));
    if (z) {
        std::memcpy(ci, g_last->get_column_index(), sizeof(int) * (size_t)z);
        std::memcpy(v, g_last->get_value(), sizeof(double) * (size_t)z);
    }
}

/* Save the last read matrix with save_pp / save_mm / save_bin. */
int ref_save(const char *fmt, const char *fn) {
    if (!g_last) return 1;
    std::string f(fmt);
    if (f == "pp") g_last->save_pp(fn);
    else if (f == "mm") g_last->save_mm(fn);
    else if (f == "bin") g_last->save_bin(fn);
    else return 1;
    return 0;
}

} // extern "C"
