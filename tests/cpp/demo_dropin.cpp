// Drop-in check: the reference demo's calls (demo/HLanc_demo.cu,
// demo/HLanc_solver_gpu.cu) compiled unchanged against include/HLanc.hpp.
// Usage: demo_dropin <pp-or-mm-or-bin> <matrix file> <nev> <ncv> [eigs file]
// With an eigs file the first solve's pairs are written in the demo's text
// format (demo/HLanc_solver_gpu.cu:57-66) and read back (demo/verify_eigs.cu).
#include <cstdio>
#include <cstdlib>

#include "HLanc.hpp"

#define N_SIMPLE 16
void op_fun_simple(double const *x, double *y) {
    for (int i = 0; i < N_SIMPLE; ++i) {
        double s = 0.0;
        for (int j = 0; j < N_SIMPLE; ++j) s += ((i < j ? i : j) + 1) * x[j];
        y[i] = s;
    }
}

template <typename op_t> struct dcsrmv_wrapper_t {
    dcsrmv_wrapper_t(op_t const &op) : op(op), seq(0) {}
    void operator()(double const *x, double *y) const {
        ++seq;
        op(x, y);
    }
    op_t const &op;
    mutable int seq;
};

int main(int argc, char *argv[]) {
    if (argc != 5 && argc != 6) {
        HLanc::warn("Usage: %s <bin|mm|pp> <matrix_file> <nev> <ncv> [eigs_file]\n", argv[0]);
        return 2;
    }
    HLanc::dcsr_matrix_t m(argv[1], argv[2]);
    int n = m.get_num_rows(), nev = atoi(argv[3]), ncv = atoi(argv[4]);
    HLanc::dcsrmv_operator_gpu op(m);
    double *values = new double[ncv];
    double *vectors = new double[(size_t)n * ncv];
    int ret = HLanc::ds_solver_gpu(n, nev, ncv, values, vectors, n, op);
    printf("device %d", ret);
    for (int i = 0; i < nev; ++i) printf(" %.15e", values[i]);
    printf("\n");
    if (argc == 6) {
        if (HLanc::write_eigs(argv[5], nev, n, values, vectors, n) != 0) return 3;
        HLanc::eigs_t eigs(argv[5]);
        printf("eigs %d %d %d\n", ret, eigs.nev, eigs.n);
    }
    // wrapped operator -> host-functor path, like demo/HLanc_solver_gpu.cu
    dcsrmv_wrapper_t<HLanc::dcsrmv_operator_gpu> wrapped(op);
    ret = HLanc::ds_solver_gpu(n, nev, ncv, values, vectors, n, wrapped);
    printf("functor %d %d", ret, wrapped.seq > 0);
    for (int i = 0; i < nev; ++i) printf(" %.15e", values[i]);
    printf("\n");
    // plain function operator (demo/HLanc_demo.cu:153-179)
    double v16[12], x16[16 * 12];
    ret = HLanc::ds_solver_gpu(N_SIMPLE, 4, 12, v16, x16, N_SIMPLE, op_fun_simple);
    printf("function %d", ret);
    for (int i = 0; i < 4; ++i) printf(" %.15e", v16[i]);
    printf("\n");
    delete[] values;
    delete[] vectors;
    return 0;
}
