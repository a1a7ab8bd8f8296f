// HLanc.hpp -- drop-in C++ API of the GB300 (sm_103a) IRLM library.
//
// Source-compatible with the reference header (butterfly0923/HLanc,
// HLanc.hpp): namespace HLanc with dcsr_matrix_t, dcsrmv_operator_gpu,
// dcsrmv_operator_naive, ds_solver_gpu<op_t>, SAFE_CALL, error_exit, warn.
// The CSR container and its pp/mm/bin readers/writers are header-only C++
// (bit-exact with the reference's); everything on the GPU goes through the C
// ABI in hlanc_gb300.h (link with -lhlanc_gb300).  No MKL, cuSPARSE or cuBLAS.
//
// ds_solver_gpu dispatches on the operator type: a dcsrmv_operator_gpu runs
// the whole implicitly restarted Lanczos loop on the device; any other
// callable (a functor, a plain function) is invoked on host vectors exactly as
// the reference invokes it, with the rest of the algorithm on the device.
#pragma once

#include <cctype>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include "hlanc_gb300.h"

#define HLANC_VERSION_MAJOR 1
#define HLANC_VERSION_MINOR 0
#define HLANC_GB300 1

#ifndef CEIL_DIV
#define CEIL_DIV(a, b) (((a) + (b)-1) / (b))
#endif
#ifndef MIN
#define MIN(a, b) ((a) < (b) ? (a) : (b))
#endif
#ifndef MAX
#define MAX(a, b) ((a) > (b) ? (a) : (b))
#endif

namespace HLanc {

// ---- utils (reference HLanc.hpp:38-67) ---------------------------------------
// Like the reference, a failing call prints file:line and exits with its
// status.  The C ABI underneath never exits; only this façade does.
template <typename status_t>
inline void check_call(status_t error, char const *file, size_t line, char const *call) {
    if (0 == (int)error) return;
    fprintf(stderr, "%s failed in \"%s:%lu\": %d (%s)\n", call, file, (unsigned long)line, (int)error,
            hlanc_status_string((int)error));
    exit((int)error);
}
#define SAFE_CALL(call) HLanc::check_call((call), __FILE__, __LINE__, #call)

inline void error_exit(char const *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stderr, fmt, ap);
    va_end(ap);
    exit(1);
}

inline void warn(char const *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stderr, fmt, ap);
    va_end(ap);
}

// ---- dcsr_matrix_t (reference HLanc.hpp:74-392) ---------------------------------
class dcsr_matrix_t {
public:
    // Reads "pp", "mm" or "bin"; on error prints a message and exits (as the
    // reference does).  Use load() for a status-returning read.
    dcsr_matrix_t(char const *format, char const *filename, bool is_symmetric = false) {
        int rc = load(format, filename, is_symmetric, true);
        if (rc) error_exit("Error reading %s file %s (status %d)\n", format, filename, rc);
    }
    // In-memory construction (extension).
    dcsr_matrix_t(int num_rows, int num_columns, std::vector<int> row_ptr, std::vector<int> column_index,
                  std::vector<double> value, bool is_symmetric = false)
        : csr_row_ptr(std::move(row_ptr)), csr_column_index(std::move(column_index)),
          csr_value(std::move(value)), num_columns(num_columns), is_symmetric(is_symmetric) {
        if ((int)csr_row_ptr.size() != num_rows + 1) error_exit("dcsr_matrix_t: row_ptr size mismatch\n");
    }
    dcsr_matrix_t() : num_columns(0), is_symmetric(false) { csr_row_ptr.push_back(0); }
    ~dcsr_matrix_t() {}

    // Status-returning reader: 0 or HLANC_ERR_IO.  verbose prints the
    // reference's "Ignore element" warnings for dropped upper entries.
    int load(char const *format, char const *filename, bool is_symmetric = false, bool verbose = false) {
        if (!strcmp(format, "pp")) return read_pp(filename, is_symmetric, verbose);
        if (!strcmp(format, "mm")) return read_mm(filename, verbose);
        if (!strcmp(format, "bin")) return read_bin(filename);
        return HLANC_ERR_IO;
    }

    void save_pp(char const *filename) const { if (write_pp(filename)) error_exit("Error writing file %s\n", filename); }
    void save_mm(char const *filename) const { if (write_mm(filename)) error_exit("Error writing file %s\n", filename); }
    void save_bin(char const *filename) const { if (write_bin(filename)) error_exit("Error writing file %s\n", filename); }

    int get_num_rows() const { return (int)csr_row_ptr.size() - 1; }
    int get_nnz() const { return (int)csr_value.size(); }
    int get_num_columns() const { return num_columns; }
    int const *get_row_ptr() const { return csr_row_ptr.data(); }
    int const *get_column_index() const { return csr_column_index.data(); }
    double const *get_value() const { return csr_value.data(); }
    bool symmetric() const { return is_symmetric; }

    // pp: "col:val" tokens separated by blanks, a row per '\n'.  Zero values
    // are dropped; with is_symmetric entries above the diagonal are dropped
    // and num_columns grows to cover the row index.  A last row without '\n'
    // leaves its entries in col/val but adds no row (reference behaviour).
    int read_pp(char const *filename, bool sym, bool verbose = false) {
        FILE *fp = fopen(filename, "r");
        if (!fp) return HLANC_ERR_IO;
        std::vector<int> rp(1, 0), ci;
        std::vector<double> va;
        int ncol = 0, rc = 0;
        for (;;) {
            int ch = fgetc(fp);
            while (ch == ' ' || ch == '\t') ch = fgetc(fp);
            if (ch == '\n') { rp.push_back((int)va.size()); continue; }
            if (ch == EOF) break;
            ungetc(ch, fp);
            int index;
            double value;
            if (fscanf(fp, "%d:%lf", &index, &value) != 2) { rc = HLANC_ERR_IO; break; }
            if (value == 0.0) continue;
            const int row = (int)rp.size() - 1;
            if (sym && index > row) {
                if (verbose) warn("Ignore element [%d, %d] = %lg\n", row, index, value);
            } else {
                ci.push_back(index);
                va.push_back(value);
            }
            if (ncol < index) ncol = index;
            if (sym && ncol < row) ncol = row;
        }
        fclose(fp);
        if (rc) return rc;
        csr_row_ptr.swap(rp);
        csr_column_index.swap(ci);
        csr_value.swap(va);
        num_columns = ncol + 1;
        is_symmetric = sym;
        return 0;
    }

    // MatrixMarket coordinate: banner decides symmetric/general, 1-based
    // indices, zeros dropped, per-row file order kept, symmetric files keep
    // col <= row.
    int read_mm(char const *filename, bool verbose = false) {
        FILE *fp = fopen(filename, "r");
        if (!fp) return HLANC_ERR_IO;
        char banner[4096];
        if (!fgets(banner, sizeof banner, fp) ||
            strncmp(banner, "%%MatrixMarket matrix coordinate", 32) != 0) {
            fclose(fp);
            return HLANC_ERR_IO;
        }
        bool sym;
        if (strstr(banner, "symmetric")) sym = true;
        else if (strstr(banner, "general")) sym = false;
        else { fclose(fp); return HLANC_ERR_IO; }
        int ch;
        while ((ch = fgetc(fp)) == '%')
            while ((ch = fgetc(fp)) != '\n' && ch != EOF) {}
        if (ch != EOF) ungetc(ch, fp);
        int rows, columns, entries;
        if (fscanf(fp, "%d%d%d", &rows, &columns, &entries) != 3 || rows < 0 || entries < 0) {
            fclose(fp);
            return HLANC_ERR_IO;
        }
        std::vector<std::vector<int> > rc_(rows);
        std::vector<std::vector<double> > rv_(rows);
        for (int q = 0; q < entries; ++q) {
            int r, c;
            double v;
            if (fscanf(fp, "%d%d%lf", &r, &c, &v) != 3) { fclose(fp); return HLANC_ERR_IO; }
            if (v == 0.0) continue;
            --r; --c;
            if (r < 0 || r >= rows) { fclose(fp); return HLANC_ERR_IO; }
            rc_[r].push_back(c);
            rv_[r].push_back(v);
        }
        fclose(fp);
        std::vector<int> rp(1, 0), ci;
        std::vector<double> va;
        for (int r = 0; r < rows; ++r) {
            for (size_t q = 0; q < rc_[r].size(); ++q) {
                if (sym && rc_[r][q] > r) {
                    if (verbose) warn("Ignore element [%d, %d] = %lg\n", r, rc_[r][q], rv_[r][q]);
                    continue;
                }
                ci.push_back(rc_[r][q]);
                va.push_back(rv_[r][q]);
            }
            rp.push_back((int)va.size());
        }
        csr_row_ptr.swap(rp);
        csr_column_index.swap(ci);
        csr_value.swap(va);
        num_columns = columns;
        is_symmetric = sym;
        return 0;
    }

    // bin: [int ncols][int nrows][int row_ptr[nrows+1]][int nnz][int col[nnz]][double val[nnz]]
    int read_bin(char const *filename) {
        FILE *fp = fopen(filename, "rb");
        if (!fp) return HLANC_ERR_IO;
        int ncol, nrow, nnz;
        int rc = HLANC_ERR_IO;
        std::vector<int> rp, ci;
        std::vector<double> va;
        if (fread(&ncol, sizeof(int), 1, fp) == 1 && fread(&nrow, sizeof(int), 1, fp) == 1 && nrow >= 0) {
            rp.resize((size_t)nrow + 1);
            if (fread(rp.data(), sizeof(int), rp.size(), fp) == rp.size() &&
                fread(&nnz, sizeof(int), 1, fp) == 1 && nnz >= 0) {
                ci.resize(nnz);
                va.resize(nnz);
                if (fread(ci.data(), sizeof(int), ci.size(), fp) == ci.size() &&
                    fread(va.data(), sizeof(double), va.size(), fp) == va.size())
                    rc = 0;
            }
        }
        fclose(fp);
        if (rc) return rc;
        csr_row_ptr.swap(rp);
        csr_column_index.swap(ci);
        csr_value.swap(va);
        num_columns = ncol;
        is_symmetric = false;
        return 0;
    }

    int write_pp(char const *filename) const {
        FILE *fp = fopen(filename, "w");
        if (!fp) return HLANC_ERR_IO;
        for (int r = 0; r + 1 < (int)csr_row_ptr.size(); ++r)
            for (int i = csr_row_ptr[r]; i < csr_row_ptr[r + 1]; ++i)
                if (fprintf(fp, "%d:%lg%c", csr_column_index[i], csr_value[i], i + 1 == csr_row_ptr[r + 1] ? '\n' : ' ') < 0) {
                    fclose(fp);
                    return HLANC_ERR_IO;
                }
        fclose(fp);
        return 0;
    }

    int write_mm(char const *filename) const {
        FILE *fp = fopen(filename, "w");
        if (!fp) return HLANC_ERR_IO;
        int rc = 0;
        if (fprintf(fp, "%%%%MatrixMarket matrix coordinate real %s\n", is_symmetric ? "symmetric" : "general") < 0 ||
            fprintf(fp, "%d %d %d\n", get_num_rows(), num_columns, get_nnz()) < 0)
            rc = HLANC_ERR_IO;
        for (int r = 0; !rc && r < get_num_rows(); ++r)
            for (int i = csr_row_ptr[r]; i < csr_row_ptr[r + 1]; ++i)
                if (fprintf(fp, "%d %d %lg\n", r + 1, csr_column_index[i] + 1, csr_value[i]) < 0) {
                    rc = HLANC_ERR_IO;
                    break;
                }
        fclose(fp);
        return rc;
    }

    // General CSR of this matrix: a symmetric (lower-stored) matrix gets each
    // off-diagonal entry mirrored; row r lists its entries in the order the
    // reference's save_bin appends them (HLanc.hpp:339-364).
    void expand_general(std::vector<int> &rp, std::vector<int> &ci, std::vector<double> &va) const {
        const int n = get_num_rows();
        rp.assign((size_t)n + 1, 0);
        for (int r = 0; r < n; ++r)
            for (int i = csr_row_ptr[r]; i < csr_row_ptr[r + 1]; ++i) {
                ++rp[r + 1];
                const int c = csr_column_index[i];
                if (is_symmetric && r != c && c >= 0 && c < n) ++rp[c + 1];
            }
        for (int r = 0; r < n; ++r) rp[r + 1] += rp[r];
        ci.assign(rp[n], 0);
        va.assign(rp[n], 0.0);
        std::vector<int> cur(rp.begin(), rp.end() - 1);
        for (int r = 0; r < n; ++r)
            for (int i = csr_row_ptr[r]; i < csr_row_ptr[r + 1]; ++i) {
                const int c = csr_column_index[i];
                const double v = csr_value[i];
                int p = cur[r]++;
                ci[p] = c;
                va[p] = v;
                if (is_symmetric && r != c && c >= 0 && c < n) {
                    p = cur[c]++;
                    ci[p] = r;
                    va[p] = v;
                }
            }
    }

    int write_bin(char const *filename) const {
        std::vector<int> rp, ci;
        std::vector<double> va;
        expand_general(rp, ci, va);
        FILE *fp = fopen(filename, "wb");
        if (!fp) return HLANC_ERR_IO;
        const int nrow = get_num_rows(), nnz = (int)ci.size();
        const bool ok = fwrite(&num_columns, sizeof(int), 1, fp) == 1 && fwrite(&nrow, sizeof(int), 1, fp) == 1 &&
                        fwrite(rp.data(), sizeof(int), rp.size(), fp) == rp.size() &&
                        fwrite(&nnz, sizeof(int), 1, fp) == 1 &&
                        fwrite(ci.data(), sizeof(int), ci.size(), fp) == ci.size() &&
                        fwrite(va.data(), sizeof(double), va.size(), fp) == va.size();
        fclose(fp);
        return ok ? 0 : HLANC_ERR_IO;
    }

protected:
    std::vector<int> csr_row_ptr;
    std::vector<int> csr_column_index;
    std::vector<double> csr_value;
    int num_columns;
    bool is_symmetric;
};

// ---- dcsrmv_operator_naive (reference HLanc.hpp:399-434) --------------------------
class dcsrmv_operator_naive {
public:
    dcsrmv_operator_naive(dcsr_matrix_t const &m) : m(m) {}
    ~dcsrmv_operator_naive() {}
    void operator()(double const *x, double *y) const {
        const int n = m.get_num_rows();
        const int *rp = m.get_row_ptr();
        const int *ci = m.get_column_index();
        const double *va = m.get_value();
        if (m.symmetric()) {
            for (int i = 0; i < n; ++i) y[i] = 0.0;
            for (int r = 0; r < n; ++r)
                for (int i = rp[r]; i < rp[r + 1]; ++i) {
                    y[r] += x[ci[i]] * va[i];
                    if (r != ci[i]) y[ci[i]] += x[r] * va[i];
                }
        } else {
            for (int r = 0; r < n; ++r) {
                double s = 0.0;
                for (int i = rp[r]; i < rp[r + 1]; ++i) s += x[ci[i]] * va[i];
                y[r] = s;
            }
        }
    }

protected:
    dcsr_matrix_t const &m;
};

// ---- dcsrmv_operator_gpu (reference HLanc.hpp:476-572) ----------------------------
// Owns a device copy of the matrix (general CSR; a symmetric matrix is
// expanded on construction).  Keeps a reference to m like the reference.
class dcsrmv_operator_gpu {
public:
    dcsrmv_operator_gpu(dcsr_matrix_t const &m, int dev = 0, int precision = HLANC_PREC_FP64)
        : m(m), dev(dev), h(nullptr) {
        SAFE_CALL(hlanc_csr_create(dev, m.get_num_rows(), m.get_num_columns(), m.get_nnz(), m.get_row_ptr(),
                                   m.get_column_index(), m.get_value(), m.symmetric() ? 1 : 0, precision, &h));
    }
    ~dcsrmv_operator_gpu() {
        if (h) hlanc_csr_destroy(h);
    }
    dcsrmv_operator_gpu(dcsrmv_operator_gpu const &) = delete;
    dcsrmv_operator_gpu &operator=(dcsrmv_operator_gpu const &) = delete;

    // y = A x; x and y may be host pointers or device pointers on `dev`.
    void operator()(double const *x, double *y) const { SAFE_CALL(hlanc_csr_apply(h, x, y)); }

    hlanc_csr_t handle() const { return h; }
    int device() const { return dev; }
    dcsr_matrix_t const &matrix() const { return m; }

protected:
    dcsr_matrix_t const &m;
    int dev;
    hlanc_csr_t h;
};

// ---- eigenpair text files -----------------------------------------------------------
// The format the reference demo writes (demo/HLanc_solver_gpu.cu:57-66) and its
// verifier reads (demo/verify_eigs.cu:8-44): nev, n, the nev eigenvalues, then
// n rows of nev vector entries, every number as "%23.15lE".
inline int write_eigs(FILE *fp, int nev, int n, double const *values, double const *vectors, int ldv) {
    if (!fp || nev < 0 || n < 0 || (nev > 0 && (!values || (n > 0 && (!vectors || ldv < n)))))
        return HLANC_ERR_INVALID;
    if (fprintf(fp, "%d\n%d\n", nev, n) < 0) return HLANC_ERR_IO;
    for (int i = 0; i < nev; ++i)
        if (fprintf(fp, "%23.15lE\n", values[i]) < 0) return HLANC_ERR_IO;
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < nev; ++c)
            if (fprintf(fp, "%23.15lE%c", vectors[r + (size_t)c * ldv], c + 1 == nev ? '\n' : ' ') < 0)
                return HLANC_ERR_IO;
    return HLANC_OK;
}

inline int write_eigs(char const *filename, int nev, int n, double const *values, double const *vectors, int ldv) {
    FILE *fp = filename ? fopen(filename, "w") : nullptr;
    if (!fp) return HLANC_ERR_IO;
    int rc = write_eigs(fp, nev, n, values, vectors, ldv);
    if (fclose(fp) != 0 && rc == HLANC_OK) rc = HLANC_ERR_IO;
    return rc;
}

// Reader of that format; vectors are stored column-major with ld n.  The
// constructor exits on errors like the reference demo's eigs_t; load()
// returns a status instead.
struct eigs_t {
    int nev = 0, n = 0;
    std::vector<double> value, vector;

    eigs_t() = default;
    explicit eigs_t(char const *filename) {
        const int rc = load(filename);
        if (rc != HLANC_OK) {
            warn("Error reading eigenpairs from \"%s\" (%s).\n", filename, hlanc_status_string(rc));
            exit(1);
        }
    }
    int load(char const *filename) {
        FILE *fp = filename ? fopen(filename, "r") : nullptr;
        if (!fp) return HLANC_ERR_IO;
        int rc = HLANC_OK;
        if (fscanf(fp, "%d", &nev) != 1 || fscanf(fp, "%d", &n) != 1 || nev < 0 || n < 0) {
            rc = HLANC_ERR_IO;
        } else {
            value.assign(nev, 0.0);
            vector.assign((size_t)n * nev, 0.0);
            for (int i = 0; i < nev && rc == HLANC_OK; ++i)
                if (fscanf(fp, "%lE", &value[i]) != 1) rc = HLANC_ERR_IO;
            for (int r = 0; r < n && rc == HLANC_OK; ++r)
                for (int c = 0; c < nev && rc == HLANC_OK; ++c)
                    if (fscanf(fp, "%lE", &vector[(size_t)c * n + r]) != 1) rc = HLANC_ERR_IO;
        }
        fclose(fp);
        if (rc != HLANC_OK) { nev = n = 0; value.clear(); vector.clear(); }
        return rc;
    }
};

template <typename T> struct is_device_csr_operator : std::false_type {};
template <> struct is_device_csr_operator<dcsrmv_operator_gpu> : std::true_type {};

namespace detail {
template <typename op_t> struct host_op_holder {
    op_t const &op;
};
template <typename op_t> int host_op_trampoline(void *ctx, const double *x, double *y) {
    static_cast<host_op_holder<op_t> *>(ctx)->op(x, y);
    return 0;
}
}  // namespace detail

// ---- ds_solver_gpu (reference HLanc.hpp:1868-1872) ----------------------------------
// Extended form: options (tolerance, restart limit, precision, start vector,
// stream) and statistics.  Returns 0 on success, 1 when fewer than nev Ritz
// values converged (the reference's failure return), >= 2 for other errors.
template <typename dspmv_operator_t>
int ds_solver_gpu_ex(int n, int nev, int ncv, double *values, double *vectors, int ldv,
                     dspmv_operator_t const &op, int dev, hlanc_opts_t const &opts,
                     hlanc_stats_t *stats = nullptr) {
    typedef typename std::remove_cv<typename std::remove_reference<dspmv_operator_t>::type>::type op_t;
    if constexpr (is_device_csr_operator<op_t>::value) {
        return hlanc_solve(dev, n, nev, ncv, values, vectors, ldv, op.handle(), nullptr, nullptr, &opts, stats);
    } else {
        detail::host_op_holder<dspmv_operator_t> holder{op};
        return hlanc_solve(dev, n, nev, ncv, values, vectors, ldv, nullptr,
                           &detail::host_op_trampoline<dspmv_operator_t>, &holder, &opts, stats);
    }
}

template <typename dspmv_operator_t>
int ds_solver_gpu(int n, int nev, int ncv, double *values, double *vectors, int ldv,
                  dspmv_operator_t const &dspmv_operator, int dev = 0) {
    hlanc_opts_t opts;
    hlanc_opts_default(&opts);
    return ds_solver_gpu_ex(n, nev, ncv, values, vectors, ldv, dspmv_operator, dev, opts, nullptr);
}

}  // namespace HLanc
