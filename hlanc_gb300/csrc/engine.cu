// engine.cu -- host side of the GB300 IRLM library and its C ABI.
//
// The implicitly restarted Lanczos loop of the reference (ds_solver,
// HLanc.hpp:1650-1850) runs here as a launch sequence per restart cycle:
//
//     [basis update]  np x [SpMV, proj, apply, proj, apply, proj, apply]  restart
//
// over every active problem of an Engine (one problem for ds_solver_gpu, many
// for a batch or the serving loop).  The sequence needs no host
// synchronisation; the host reads the problems' State structs once per cycle
// (a few hundred bytes) to learn nev/np for the next cycle and to retire
// finished problems.  Identical cycles are replayed as CUDA graphs.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "../../include/HLanc.hpp"
#include "internal.cuh"

using namespace hlanc;

// ------------------------------------------------------------------------------
#define CK(x)                                                      \
    do {                                                           \
        cudaError_t e_ = (x);                                      \
        if (e_ != cudaSuccess) {                                   \
            report_cuda_error(e_, #x, __FILE__, __LINE__);         \
            return HLANC_ERR_CUDA;                                 \
        }                                                          \
    } while (0)

static void report_cuda_error(cudaError_t e, const char *what, const char *file, int line) {
    if (getenv("HLANC_VERBOSE"))
        fprintf(stderr, "hlanc: %s failed at %s:%d: %s\n", what, file, line, cudaGetErrorString(e));
}

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---- device CSR operator --------------------------------------------------------
struct hlanc_csr_s {
    int dev = 0, nrows = 0, ncols = 0, precision = HLANC_PREC_FP64;
    long long nnz = 0;
    int *rp_d = nullptr, *ci_d = nullptr;
    double *val_d = nullptr;
    float *val32_d = nullptr;
    double *xs_d = nullptr, *ys_d = nullptr;   // staging for host vectors (HLanc.hpp:541-549)
    cudaStream_t stream = nullptr;
    double norm_inf = 0.0;                      // max_r sum |a_rc|
    std::mutex mu;
};

struct hlanc_matrix_s {
    HLanc::dcsr_matrix_t m;
};

namespace {

struct DevGuard {
    int prev = -1;
    explicit DevGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DevGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

int tile_rows_for(int n) {
    long long tr = ((long long)n + 1215) / 1216;         // ~1216 tiles per large problem
    tr = (tr + ROW_ALIGN - 1) / ROW_ALIGN * ROW_ALIGN;
    if (tr < 128) tr = 128;
    if (tr > 8192) tr = 8192;
    return (int)tr;
}

// ---- one problem's device resources ---------------------------------------------
struct ProbRes {
    int n = 0, ncv = 0, nev0 = 0, ld = 0, ntiles = 0, tr = 0, pstride = 0;
    int fp32 = 0;
    hlanc_csr_s *csr = nullptr;
    hlanc_host_op_fn host_op = nullptr;
    void *host_ctx = nullptr;
    double *block = nullptr;       // V | r0 | r1 | part | small
    double *V = nullptr, *r0 = nullptr, *r1 = nullptr, *part = nullptr, *small = nullptr;
    State *st = nullptr;
    unsigned *counter = nullptr;
    float *x32 = nullptr;
    double *vout = nullptr;
    int ldo = 0;
    bool own_vout = false;
    size_t bytes = 0;

    static size_t estimate(int n, int ncv, int fp32) {
        const int ld = (n + ROW_ALIGN - 1) / ROW_ALIGN * ROW_ALIGN;
        const int tr = tile_rows_for(n);
        const int ntiles = (n + tr - 1) / tr;
        const int pst = (ncv + 2 + 1) & ~1;
        size_t d = (size_t)ld * ncv + 2 * (size_t)ld + (size_t)ntiles * pst + SM_SIZE(ncv);
        size_t b = d * sizeof(double) + sizeof(State) + 256;
        if (fp32) b += (size_t)ld * sizeof(float);
        b += (size_t)ld * ncv * sizeof(double);   // Ritz output
        return b;
    }

    int alloc(cudaStream_t s) {
        ld = (n + ROW_ALIGN - 1) / ROW_ALIGN * ROW_ALIGN;
        tr = tile_rows_for(n);
        ntiles = (n + tr - 1) / tr;
        pstride = (ncv + 2 + 1) & ~1;
        const size_t nd = (size_t)ld * ncv + 2 * (size_t)ld + (size_t)ntiles * pstride + SM_SIZE(ncv);
        bytes = nd * sizeof(double);
        CK(cudaMalloc(&block, bytes));
        CK(cudaMemsetAsync(block, 0, bytes, s));
        V = block;
        r0 = V + (size_t)ld * ncv;
        r1 = r0 + ld;
        part = r1 + ld;
        small = part + (size_t)ntiles * pstride;
        void *sp = nullptr;
        CK(cudaMalloc(&sp, sizeof(State) + 256));
        CK(cudaMemsetAsync(sp, 0, sizeof(State) + 256, s));
        st = (State *)sp;
        counter = (unsigned *)((char *)sp + sizeof(State) + 64);
        if (fp32) {
            CK(cudaMalloc(&x32, (size_t)ld * sizeof(float)));
            CK(cudaMemsetAsync(x32, 0, (size_t)ld * sizeof(float), s));
            bytes += (size_t)ld * sizeof(float);
        }
        return HLANC_OK;
    }
    void release() {
        if (block) cudaFree(block);
        if (st) cudaFree(st);
        if (x32) cudaFree(x32);
        if (own_vout && vout) cudaFree(vout);
        block = nullptr; st = nullptr; x32 = nullptr; vout = nullptr;
    }
};

State initial_state(int nev, int ncv, const hlanc_opts_t &o) {
    State S;
    memset(&S, 0, sizeof S);
    S.status = ST_RUNNING;
    S.phase = PH_EXTEND;
    S.k = 0;
    S.np = ncv;          // the first extension runs steps 0..ncv-1 (HLanc.hpp:1680 + 1685)
    S.nev = nev;
    S.iter = -1;         // start-vector norm pending
    S.max_iter = o.max_restarts > 0 ? o.max_restarts : 200;
    S.nev0 = nev;
    S.np0 = ncv - nev;
    S.ncv = ncv;
    const double eps = 1.1102230246251565e-16;   // dlamch("E") = 2^-53
    S.tol = o.tol > 0.0 ? o.tol : eps;
    S.eps23 = pow(eps, 0.66666666666666663);      // HLanc.hpp:1652
    return S;
}

// ---- the engine: a set of problems sharing launches ------------------------------
class Engine {
public:
    int dev = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool use_graphs = true;
    std::vector<ProbRes> probs;
    std::vector<int> active;            // indices of problems in the launch tables
    Problem *P_d = nullptr;
    Tile *T_d = nullptr;
    int ntiles = 0, nslots = 0;
    State *st_h = nullptr;              // pinned mirror of every problem's State
    int st_cap = 0;
    int max_ncv = 0, max_nev0 = 0;
    bool fp32_any = false;
    std::map<long long, cudaGraphExec_t> graphs;
    double *xs_h = nullptr, *ys_h = nullptr, *xs_d = nullptr;   // host-operator staging
    size_t xs_cap = 0;

    ~Engine() {
        DevGuard g(dev);
        drop_graphs();
        for (auto &p : probs) p.release();
        if (P_d) cudaFree(P_d);
        if (T_d) cudaFree(T_d);
        if (st_h) cudaFreeHost(st_h);
        if (xs_h) cudaFreeHost(xs_h);
        if (ys_h) cudaFreeHost(ys_h);
        if (xs_d) cudaFree(xs_d);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }

    int init(int device, void *user_stream, bool graphs_on) {
        dev = device;
        use_graphs = graphs_on;
        if (user_stream) {
            stream = (cudaStream_t)user_stream;
        } else {
            CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
            own_stream = true;
        }
        return HLANC_OK;
    }

    void drop_graphs() {
        for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
    }

    int add(int n, int nev, int ncv, hlanc_csr_s *csr, hlanc_host_op_fn host_op, void *host_ctx,
            int fp32, const hlanc_opts_t &o, int *index) {
        ProbRes p;
        p.n = n; p.ncv = ncv; p.nev0 = nev; p.csr = csr; p.host_op = host_op; p.host_ctx = host_ctx;
        p.fp32 = fp32;
        int rc = p.alloc(stream);
        if (rc) { p.release(); return rc == HLANC_ERR_CUDA ? HLANC_ERR_ALLOC : rc; }
        State S = initial_state(nev, ncv, o);
        CK(cudaMemcpyAsync(p.st, &S, sizeof S, cudaMemcpyHostToDevice, stream));
        probs.push_back(p);
        *index = (int)probs.size() - 1;
        return HLANC_OK;
    }

    // Rebuild the device descriptor and tile tables for the problems in `active`.
    int upload() {
        std::vector<Problem> P(active.size());
        std::vector<Tile> T;
        max_ncv = 0; max_nev0 = 0; fp32_any = false;
        for (size_t a = 0; a < active.size(); ++a) {
            ProbRes &p = probs[active[a]];
            Problem &q = P[a];
            memset(&q, 0, sizeof q);
            if (p.csr) {
                q.row_ptr = p.csr->rp_d; q.col = p.csr->ci_d; q.val = p.csr->val_d;
                q.val32 = p.fp32 ? p.csr->val32_d : nullptr;
            }
            q.x32 = p.x32;
            q.n = p.n; q.ld = p.ld; q.ncv = p.ncv; q.nev0 = p.nev0;
            q.tile0 = (int)T.size(); q.ntiles = p.ntiles;
            q.fp32 = p.fp32; q.pstride = p.pstride;
            q.V = p.V; q.r0 = p.r0; q.r1 = p.r1; q.part = p.part; q.counter = p.counter;
            q.st = p.st; q.small = p.small;
            q.wext = p.csr ? nullptr : p.r0;     // non-null marks the host-operator path
            q.vout = p.vout; q.ldo = p.ldo;
            for (int t = 0; t < p.ntiles; ++t) {
                Tile tl;
                tl.prob = (int)a;
                tl.row0 = t * p.tr;
                tl.row1 = std::min(p.n, (t + 1) * p.tr);
                tl.pad = 0;
                T.push_back(tl);
            }
            max_ncv = std::max(max_ncv, p.ncv);
            max_nev0 = std::max(max_nev0, p.nev0);
            fp32_any = fp32_any || p.fp32;
        }
        if ((int)active.size() > nslots || (int)T.size() > ntiles || !P_d || !T_d) {
            if (P_d) cudaFree(P_d);
            if (T_d) cudaFree(T_d);
            nslots = std::max<int>((int)active.size(), 1);
            CK(cudaMalloc(&P_d, sizeof(Problem) * nslots));
            CK(cudaMalloc(&T_d, sizeof(Tile) * std::max<size_t>(T.size(), 1)));
        }
        ntiles = (int)T.size();
        if (!P.empty()) CK(cudaMemcpyAsync(P_d, P.data(), sizeof(Problem) * P.size(), cudaMemcpyHostToDevice, stream));
        if (!T.empty()) CK(cudaMemcpyAsync(T_d, T.data(), sizeof(Tile) * T.size(), cudaMemcpyHostToDevice, stream));
        if ((int)active.size() > st_cap) {
            if (st_h) cudaFreeHost(st_h);
            st_cap = (int)active.size() + 8;
            CK(cudaMallocHost(&st_h, sizeof(State) * st_cap));
        }
        drop_graphs();
        return HLANC_OK;
    }

    int slot_of(int prob) const {
        for (size_t a = 0; a < active.size(); ++a)
            if (active[a] == prob) return (int)a;
        return -1;
    }

    int start_vector(int prob, const hlanc_opts_t &o) {
        ProbRes &p = probs[prob];
        if (o.start) {
            CK(cudaMemcpyAsync(p.r0, o.start, sizeof(double) * p.n, cudaMemcpyHostToDevice, stream));
        } else {
            launch_start_vector(P_d, T_d, ntiles, slot_of(prob), o.seed, stream);
        }
        launch_norm_init(P_d, T_d, ntiles, stream);
        return HLANC_OK;
    }

    int readback() {
        for (size_t a = 0; a < active.size(); ++a)
            CK(cudaMemcpyAsync(st_h + a, probs[active[a]].st, sizeof(State), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        CK(cudaGetLastError());
        return HLANC_OK;
    }

    void enqueue_cycle(int steps, int basis_nev) {
        if (basis_nev > 0) launch_basis(P_d, T_d, ntiles, max_ncv, basis_nev, stream);
        for (int s = 0; s < steps; ++s) launch_step(P_d, T_d, ntiles, s, fp32_any, false, stream);
        launch_restart(P_d, (int)active.size(), max_ncv, stream);
    }

    // One restart cycle of every active problem with a device operator.
    int run_cycle(int steps, int basis_nev) {
        if (!use_graphs) {
            enqueue_cycle(steps, basis_nev);
            CK(cudaGetLastError());
            return HLANC_OK;
        }
        const long long key = (long long)steps * 1024 + basis_nev;
        auto it = graphs.find(key);
        if (it == graphs.end()) {
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            enqueue_cycle(steps, basis_nev);
            CK(cudaStreamEndCapture(stream, &g));
            cudaGraphExec_t ge;
            cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            CK(e);
            it = graphs.emplace(key, ge).first;
        }
        CK(cudaGraphLaunch(it->second, stream));
        return HLANC_OK;
    }

    // One restart cycle of a single host-operator problem (synchronous steps).
    int run_cycle_host(int prob, int steps, int basis_nev) {
        ProbRes &p = probs[prob];
        if (xs_cap < (size_t)p.n) {
            if (xs_h) cudaFreeHost(xs_h);
            if (ys_h) cudaFreeHost(ys_h);
            if (xs_d) cudaFree(xs_d);
            CK(cudaMallocHost(&xs_h, sizeof(double) * p.n));
            CK(cudaMallocHost(&ys_h, sizeof(double) * p.n));
            CK(cudaMalloc(&xs_d, sizeof(double) * p.n));
            xs_cap = p.n;
        }
        if (basis_nev > 0) launch_basis(P_d, T_d, ntiles, max_ncv, basis_nev, stream);
        int rc = readback();
        if (rc) return rc;
        const int a = slot_of(prob);
        const int k = st_h[a].k;
        for (int s = 0; s < steps; ++s) {
            const int j = k + s;
            launch_prep_ext(P_d, T_d, ntiles, s, xs_d, stream);
            CK(cudaMemcpyAsync(xs_h, xs_d, sizeof(double) * p.n, cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            if (p.host_op(p.host_ctx, xs_h, ys_h) != 0) return HLANC_ERR_CALLBACK;
            double *w = ((j + 1) & 1) ? p.r1 : p.r0;
            CK(cudaMemcpyAsync(w, ys_h, sizeof(double) * p.n, cudaMemcpyHostToDevice, stream));
            launch_step(P_d, T_d, ntiles, s, false, true, stream);
        }
        launch_restart(P_d, (int)active.size(), max_ncv, stream);
        CK(cudaGetLastError());
        return HLANC_OK;
    }

    // Converged problem -> explicit Q factor and Ritz vectors into p.vout.
    int finalize(int prob) {
        ProbRes &p = probs[prob];
        if (!p.vout) {
            CK(cudaMalloc(&p.vout, sizeof(double) * (size_t)p.ld * p.ncv));
            p.own_vout = true;
            p.ldo = p.ld;
        }
        int rc = upload();
        if (rc) return rc;
        launch_finalize(P_d, (int)active.size(), max_ncv, stream);
        launch_ritz(P_d, T_d, ntiles, max_ncv, stream);
        CK(cudaGetLastError());
        return HLANC_OK;
    }
};

// Drive one problem (or a whole engine) to completion.  Returns per-problem
// terminal states in st_h.
int drive(Engine &E, const std::vector<int> &which) {
    // first cycle: every problem extends 0..ncv-1
    int max_steps = 0;
    for (int p : which) max_steps = std::max(max_steps, E.probs[p].ncv);
    bool host_path = false;
    for (int p : which) host_path = host_path || !E.probs[p].csr;
    int basis_nev = 0;
    int steps = max_steps;
    for (;;) {
        int rc;
        if (host_path) rc = E.run_cycle_host(which[0], steps, basis_nev);
        else rc = E.run_cycle(steps, basis_nev);
        if (rc) return rc;
        if ((rc = E.readback())) return rc;
        int running = 0, nmax = 0, stepmax = 0;
        for (size_t a = 0; a < E.active.size(); ++a) {
            const State &S = E.st_h[a];
            if (S.status == ST_RUNNING && S.phase == PH_APPLY) {
                ++running;
                nmax = std::max(nmax, S.nev);
                stepmax = std::max(stepmax, S.np);
            }
        }
        if (!running) break;
        basis_nev = nmax;
        steps = stepmax;
    }
    return HLANC_OK;
}

void fill_stats(hlanc_stats_t *stats, const State &S, const ProbRes &p, double nnz, int fp32,
                int refine_restarts, double seconds, int status) {
    if (!stats) return;
    memset(stats, 0, sizeof(*stats));
    stats->spmv_calls = S.spmv;
    stats->cgs_passes = S.passes;
    stats->restarts = S.iter;
    stats->nconv = S.nconv;
    stats->refine_restarts = refine_restarts;
    stats->status = status;
    stats->rnorm = S.rnorm;
    stats->seconds = seconds;
    const double n = p.n;
    const double spmv_b = fp32 ? (8.0 * nnz + 4.0 * (n + 1) + 8.0 * n + 16.0 * n)
                               : (12.0 * nnz + 4.0 * (n + 1) + 16.0 * n + 16.0 * n);
    stats->bytes_spmv = spmv_b * (double)S.spmv;
    stats->bytes_cgs = 16.0 * n * (double)S.sumc + 24.0 * n * (double)S.passes;
    stats->bytes_restart = (8.0 * n * p.ncv + 16.0 * n) * S.napply + 8.0 * n * (double)S.sumnev;
}

int map_status(int st) {
    switch (st) {
    case ST_CONVERGED: return HLANC_OK;
    case ST_NOT_CONVERGED: return HLANC_NOT_CONVERGED;
    case ST_FAILED: return HLANC_NOT_CONVERGED;
    default: return HLANC_NOT_CONVERGED;
    }
}

__global__ void k_sum_columns(const double *__restrict__ Y, int ld, int n, int k, double *__restrict__ out) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < k; ++i) s += Y[(size_t)i * ld + r];
        out[r] = s;
    }
}

// Full solve of one problem on an engine.  values_out/vectors_out are host
// (device_out = false) or device pointers.
int solve_one(int dev, int n, int nev, int ncv, double *values, double *vectors, int ldv, bool device_out,
              hlanc_csr_s *csr, hlanc_host_op_fn host_op, void *host_ctx, const hlanc_opts_t &o,
              hlanc_stats_t *stats) {
    const double t0 = now_s();
    DevGuard g(dev);
    Engine E;
    int rc = E.init(dev, o.stream, o.use_graphs != 0);
    if (rc) return rc;
    const bool fp32 = csr && o.precision == HLANC_PREC_FP32_REFINE && csr->val32_d;
    int idx = 0;
    // phase 1: FP32 SpMV to a loose tolerance when mixed precision is asked for
    hlanc_opts_t o1 = o;
    if (fp32) o1.tol = std::max(o.tol > 0 ? o.tol : 0.0, 1e-6);
    rc = E.add(n, nev, ncv, csr, host_op, host_ctx, fp32 ? 1 : 0, o1, &idx);
    if (rc) return rc;
    E.active = {idx};
    if ((rc = E.upload())) return rc;
    if ((rc = E.start_vector(idx, o))) return rc;
    if ((rc = drive(E, E.active))) return rc;
    State S1 = E.st_h[0];
    int refine_restarts = 0;
    State S = S1;
    if (fp32) {
        // phase 2: FP64 restarts warm-started from the sum of the FP32 Ritz vectors
        ProbRes &p = E.probs[idx];
        if (S1.status == ST_CONVERGED) {
            if ((rc = E.finalize(idx))) return rc;
            k_sum_columns<<<304, 256, 0, E.stream>>>(p.vout, p.ldo, p.n, S1.nconv, p.r0);
            launch_counter() += 1;
        }
        State S0 = initial_state(nev, ncv, o);
        CK(cudaMemcpyAsync(p.st, &S0, sizeof S0, cudaMemcpyHostToDevice, E.stream));
        p.fp32 = 0;
        if ((rc = E.upload())) return rc;
        launch_norm_init(E.P_d, E.T_d, E.ntiles, E.stream);
        if ((rc = drive(E, E.active))) return rc;
        S = E.st_h[0];
        refine_restarts = S.iter;
        S.spmv += S1.spmv;
        S.passes += S1.passes;
        S.sumc += S1.sumc;
        S.sumnev += S1.sumnev;
        S.napply += S1.napply;
    }
    int status = map_status(S.status);
    if (S.status == ST_CONVERGED) {
        ProbRes &p = E.probs[idx];
        if (device_out) {
            if (p.own_vout && p.vout) cudaFree(p.vout);
            p.vout = vectors;
            p.ldo = ldv;
            p.own_vout = false;
        }
        if ((rc = E.finalize(idx))) return rc;
        if ((rc = E.readback())) return rc;
        if (E.st_h[0].status != ST_CONVERGED) {
            status = HLANC_NOT_CONVERGED;
        } else {
            const int m = p.ncv;
            const int nconv = E.st_h[0].nconv;
            if (device_out) {
                CK(cudaMemcpyAsync(values, p.small + SM_VALS(m), sizeof(double) * nconv, cudaMemcpyDeviceToDevice, E.stream));
            } else {
                CK(cudaMemcpyAsync(values, p.small + SM_VALS(m), sizeof(double) * nconv, cudaMemcpyDeviceToHost, E.stream));
                CK(cudaMemcpy2DAsync(vectors, sizeof(double) * (size_t)ldv, p.vout, sizeof(double) * (size_t)p.ldo,
                                     sizeof(double) * (size_t)n, m, cudaMemcpyDeviceToHost, E.stream));
            }
            CK(cudaStreamSynchronize(E.stream));
        }
    }
    const double nnz = csr ? (double)csr->nnz : 0.0;
    fill_stats(stats, S, E.probs[idx], nnz, fp32 ? 1 : 0, refine_restarts, now_s() - t0, status);
    if (stats && S.status == ST_CONVERGED) stats->bytes_restart += 16.0 * n * ncv;
    return status;
}

int validate(int n, int nev, int ncv, int ldv) {
    if (n <= 0 || nev <= 0 || ncv <= nev || ncv > n || ldv < n) return HLANC_ERR_INVALID;
    if (ncv > HLANC_MAX_NCV || nev > HLANC_MAX_NEV) return HLANC_ERR_UNSUPPORTED;
    return HLANC_OK;
}

}  // namespace

// =============================================================================
// C ABI
// =============================================================================
extern "C" {

const char *hlanc_status_string(int status) {
    switch (status) {
    case HLANC_OK: return "ok";
    case HLANC_NOT_CONVERGED: return "not converged";
    case HLANC_ERR_INVALID: return "invalid argument";
    case HLANC_ERR_CUDA: return "CUDA error";
    case HLANC_ERR_ALLOC: return "allocation failed";
    case HLANC_ERR_DEVICE_TIMEOUT: return "device wait timed out";
    case HLANC_ERR_IO: return "matrix file error";
    case HLANC_ERR_UNSUPPORTED: return "unsupported size";
    case HLANC_ERR_CALLBACK: return "host operator failed";
    case HLANC_ERR_CANCELLED: return "cancelled";
    default: return "unknown status";
    }
}

int hlanc_version(int *major, int *minor) {
    if (major) *major = HLANC_VERSION_MAJOR;
    if (minor) *minor = HLANC_VERSION_MINOR;
    return HLANC_OK;
}

long long hlanc_kernel_launches(void) { return launch_counter(); }

void hlanc_opts_default(hlanc_opts_t *o) {
    memset(o, 0, sizeof(*o));
    o->tol = 0.0;
    o->max_restarts = 200;
    o->precision = HLANC_PREC_FP64;
    o->seed = 0;
    o->start = nullptr;
    o->stream = nullptr;
    o->use_graphs = 1;
}

// ---- host matrices -------------------------------------------------------------
int hlanc_matrix_read(const char *format, const char *filename, int is_symmetric, hlanc_matrix_t *out) {
    if (!format || !filename || !out) return HLANC_ERR_INVALID;
    std::unique_ptr<hlanc_matrix_s> m(new hlanc_matrix_s());
    int rc = m->m.load(format, filename, is_symmetric != 0, false);
    if (rc) return rc;
    *out = m.release();
    return HLANC_OK;
}

int hlanc_matrix_create(int nrows, int ncols, int nnz, const int *row_ptr, const int *col, const double *val,
                        int is_symmetric, hlanc_matrix_t *out) {
    if (nrows < 0 || nnz < 0 || !row_ptr || !out || (nnz > 0 && (!col || !val))) return HLANC_ERR_INVALID;
    std::vector<int> rp(row_ptr, row_ptr + nrows + 1), ci(col, col + nnz);
    std::vector<double> va(val, val + nnz);
    *out = new hlanc_matrix_s{HLanc::dcsr_matrix_t(nrows, ncols, std::move(rp), std::move(ci), std::move(va),
                                                   is_symmetric != 0)};
    return HLANC_OK;
}

int hlanc_matrix_info(hlanc_matrix_t m, int *nrows, int *ncols, int *nnz, int *is_symmetric) {
    if (!m) return HLANC_ERR_INVALID;
    if (nrows) *nrows = m->m.get_num_rows();
    if (ncols) *ncols = m->m.get_num_columns();
    if (nnz) *nnz = m->m.get_nnz();
    if (is_symmetric) *is_symmetric = m->m.symmetric() ? 1 : 0;
    return HLANC_OK;
}

int hlanc_matrix_arrays(hlanc_matrix_t m, const int **row_ptr, const int **col, const double **val) {
    if (!m) return HLANC_ERR_INVALID;
    if (row_ptr) *row_ptr = m->m.get_row_ptr();
    if (col) *col = m->m.get_column_index();
    if (val) *val = m->m.get_value();
    return HLANC_OK;
}

int hlanc_matrix_save(hlanc_matrix_t m, const char *format, const char *filename) {
    if (!m || !format || !filename) return HLANC_ERR_INVALID;
    if (!strcmp(format, "pp")) return m->m.write_pp(filename);
    if (!strcmp(format, "mm")) return m->m.write_mm(filename);
    if (!strcmp(format, "bin")) return m->m.write_bin(filename);
    return HLANC_ERR_INVALID;
}

int hlanc_matrix_destroy(hlanc_matrix_t m) {
    delete m;
    return HLANC_OK;
}

// ---- device CSR operator --------------------------------------------------------
int hlanc_csr_create(int dev, int nrows, int ncols, int nnz, const int *row_ptr, const int *col,
                     const double *val, int is_symmetric, int precision, hlanc_csr_t *out) {
    if (!out || nrows < 0 || ncols < 0 || nnz < 0 || !row_ptr || (nnz > 0 && (!col || !val)))
        return HLANC_ERR_INVALID;
    if (precision != HLANC_PREC_FP64 && precision != HLANC_PREC_FP32_REFINE) return HLANC_ERR_INVALID;
    if (row_ptr[0] != 0) return HLANC_ERR_INVALID;
    for (int r = 0; r < nrows; ++r)
        if (row_ptr[r + 1] < row_ptr[r]) return HLANC_ERR_INVALID;
    if (row_ptr[nrows] > nnz) return HLANC_ERR_INVALID;
    const int used = row_ptr[nrows];
    for (int i = 0; i < used; ++i)
        if (col[i] < 0 || col[i] >= ncols) return HLANC_ERR_INVALID;
    // general CSR on the device: symmetric-lower input is mirrored (only
    // entries with col <= row are used, as cuSPARSE SYMMETRIC / mkl "SLNC" do)
    std::vector<int> rp, ci;
    std::vector<double> va;
    const int *grp = row_ptr, *gci = col;
    const double *gva = val;
    if (is_symmetric) {
        rp.assign((size_t)nrows + 1, 0);
        for (int r = 0; r < nrows; ++r)
            for (int i = row_ptr[r]; i < row_ptr[r + 1]; ++i) {
                const int c = col[i];
                if (c > r) continue;
                ++rp[r + 1];
                if (c < r) ++rp[c + 1];
            }
        for (int r = 0; r < nrows; ++r) rp[r + 1] += rp[r];
        ci.resize(rp[nrows]);
        va.resize(rp[nrows]);
        std::vector<int> cur(rp.begin(), rp.end() - 1);
        for (int r = 0; r < nrows; ++r)
            for (int i = row_ptr[r]; i < row_ptr[r + 1]; ++i) {
                const int c = col[i];
                if (c > r) continue;
                int p = cur[r]++;
                ci[p] = c; va[p] = val[i];
                if (c < r) { p = cur[c]++; ci[p] = r; va[p] = val[i]; }
            }
        grp = rp.data(); gci = ci.data(); gva = va.data();
    }
    const long long gnnz = grp[nrows];
    std::unique_ptr<hlanc_csr_s> h(new hlanc_csr_s());
    h->dev = dev; h->nrows = nrows; h->ncols = ncols; h->precision = precision; h->nnz = gnnz;
    double ninf = 0.0;
    for (int r = 0; r < nrows; ++r) {
        double s = 0.0;
        for (int i = grp[r]; i < grp[r + 1]; ++i) s += fabs(gva[i]);
        ninf = std::max(ninf, s);
    }
    h->norm_inf = ninf;
    DevGuard g(dev);
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    const size_t nz = (size_t)std::max<long long>(gnnz, 1);
    CK(cudaMalloc(&h->rp_d, sizeof(int) * ((size_t)nrows + 1)));
    CK(cudaMalloc(&h->ci_d, sizeof(int) * nz + 16));
    CK(cudaMalloc(&h->val_d, sizeof(double) * nz + 16));
    CK(cudaMalloc(&h->xs_d, sizeof(double) * (size_t)std::max(ncols, 1)));
    CK(cudaMalloc(&h->ys_d, sizeof(double) * (size_t)std::max(nrows, 1)));
    CK(cudaMemcpyAsync(h->rp_d, grp, sizeof(int) * ((size_t)nrows + 1), cudaMemcpyHostToDevice, h->stream));
    if (gnnz) {
        CK(cudaMemcpyAsync(h->ci_d, gci, sizeof(int) * gnnz, cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->val_d, gva, sizeof(double) * gnnz, cudaMemcpyHostToDevice, h->stream));
    }
    if (precision == HLANC_PREC_FP32_REFINE) {
        std::vector<float> v32((size_t)gnnz);
        for (long long i = 0; i < gnnz; ++i) v32[i] = (float)gva[i];
        CK(cudaMalloc(&h->val32_d, sizeof(float) * nz + 16));
        if (gnnz) CK(cudaMemcpyAsync(h->val32_d, v32.data(), sizeof(float) * gnnz, cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    *out = h.release();
    return HLANC_OK;
}

int hlanc_csr_destroy(hlanc_csr_t h) {
    if (!h) return HLANC_OK;
    {
        DevGuard g(h->dev);
        cudaFree(h->rp_d); cudaFree(h->ci_d); cudaFree(h->val_d);
        if (h->val32_d) cudaFree(h->val32_d);
        cudaFree(h->xs_d); cudaFree(h->ys_d);
        if (h->stream) cudaStreamDestroy(h->stream);
    }
    delete h;
    return HLANC_OK;
}

int hlanc_csr_info(hlanc_csr_t h, int *dev, int *nrows, int *ncols, long long *nnz, int *precision) {
    if (!h) return HLANC_ERR_INVALID;
    if (dev) *dev = h->dev;
    if (nrows) *nrows = h->nrows;
    if (ncols) *ncols = h->ncols;
    if (nnz) *nnz = h->nnz;
    if (precision) *precision = h->precision;
    return HLANC_OK;
}

static bool is_device_ptr(const void *p, int dev) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

int hlanc_csr_apply(hlanc_csr_t h, const double *x, double *y) {
    if (!h || !x || !y) return HLANC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(h->mu);
    DevGuard g(h->dev);
    const double *xx = x;
    double *yy = y;
    if (!is_device_ptr(x, h->dev)) {
        CK(cudaMemcpyAsync(h->xs_d, x, sizeof(double) * h->ncols, cudaMemcpyDefault, h->stream));
        xx = h->xs_d;
    }
    if (!is_device_ptr(y, h->dev)) yy = h->ys_d;
    launch_spmv(h->rp_d, h->ci_d, h->val_d, h->nrows, xx, yy, h->stream);
    CK(cudaGetLastError());
    if (yy != y) CK(cudaMemcpyAsync(y, yy, sizeof(double) * h->nrows, cudaMemcpyDefault, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return HLANC_OK;
}

int hlanc_csr_spmv_async(hlanc_csr_t h, const double *x_d, double *y_d, void *stream) {
    if (!h || !x_d || !y_d) return HLANC_ERR_INVALID;
    DevGuard g(h->dev);
    launch_spmv(h->rp_d, h->ci_d, h->val_d, h->nrows, x_d, y_d, (cudaStream_t)stream);
    CK(cudaGetLastError());
    return HLANC_OK;
}

int hlanc_csr_spmv_f32_async(hlanc_csr_t h, const float *x_d, float *y_d, void *stream) {
    if (!h || !x_d || !y_d) return HLANC_ERR_INVALID;
    if (!h->val32_d) return HLANC_ERR_INVALID;
    DevGuard g(h->dev);
    launch_spmv_f32(h->rp_d, h->ci_d, h->val32_d, h->nrows, x_d, y_d, (cudaStream_t)stream);
    CK(cudaGetLastError());
    return HLANC_OK;
}

// ---- solver -------------------------------------------------------------------------
struct csr_cb_ctx { hlanc_csr_t h; };
static int csr_host_cb(void *ctx, const double *x, double *y) {
    return hlanc_csr_apply(static_cast<csr_cb_ctx *>(ctx)->h, x, y);
}

int hlanc_solve(int dev, int n, int nev, int ncv, double *values, double *vectors, int ldv, hlanc_csr_t csr,
                hlanc_host_op_fn host_op, void *host_ctx, const hlanc_opts_t *opts, hlanc_stats_t *stats) {
    int rc = validate(n, nev, ncv, ldv);
    if (rc) return rc;
    if (!values || !vectors) return HLANC_ERR_INVALID;
    hlanc_opts_t o;
    if (opts) o = *opts;
    else hlanc_opts_default(&o);
    csr_cb_ctx cb{csr};
    if (csr) {
        if (csr->nrows != n || csr->ncols > n) return HLANC_ERR_INVALID;
        if (csr->dev != dev) {     // operator on another device: call it like a host functor
            host_op = csr_host_cb;
            host_ctx = &cb;
            csr = nullptr;
        }
    } else if (!host_op) {
        return HLANC_ERR_INVALID;
    }
    if (!csr) o.precision = HLANC_PREC_FP64;
    return solve_one(dev, n, nev, ncv, values, vectors, ldv, false, csr, host_op, host_ctx, o, stats);
}

int hlanc_solve_device(int dev, int n, int nev, int ncv, double *values_d, double *vectors_d, int ldv_d,
                       hlanc_csr_t csr, const hlanc_opts_t *opts, hlanc_stats_t *stats) {
    int rc = validate(n, nev, ncv, ldv_d);
    if (rc) return rc;
    if (!values_d || !vectors_d || !csr) return HLANC_ERR_INVALID;
    if (csr->nrows != n || csr->ncols > n || csr->dev != dev) return HLANC_ERR_INVALID;
    hlanc_opts_t o;
    if (opts) o = *opts;
    else hlanc_opts_default(&o);
    return solve_one(dev, n, nev, ncv, values_d, vectors_d, ldv_d, true, csr, nullptr, nullptr, o, stats);
}

int hlanc_residuals_device(hlanc_csr_t csr, int k, const double *values_d, const double *vectors_d, int ldv_d,
                           double *resid_h, double *rdiff_h) {
    if (!csr || k <= 0 || !values_d || !vectors_d || ldv_d < csr->nrows) return HLANC_ERR_INVALID;
    DevGuard g(csr->dev);
    double *out = nullptr;
    CK(cudaMalloc(&out, sizeof(double) * 4 * (size_t)k));
    launch_residuals(csr->rp_d, csr->ci_d, csr->val_d, csr->nrows, k, values_d, vectors_d, ldv_d, out, csr->stream);
    std::vector<double> h(4 * (size_t)k);
    cudaError_t e = cudaMemcpyAsync(h.data(), out, sizeof(double) * 4 * k, cudaMemcpyDeviceToHost, csr->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(csr->stream);
    cudaFree(out);
    CK(e);
    for (int i = 0; i < k; ++i) {
        if (resid_h) resid_h[i] = sqrt(h[4 * i]);
        const double mx = std::max(h[4 * i + 2], h[4 * i + 3]);
        if (rdiff_h) rdiff_h[i] = mx > 0 ? h[4 * i + 1] / mx : h[4 * i + 1];
    }
    return HLANC_OK;
}

}  // extern "C"
