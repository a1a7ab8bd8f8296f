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
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/HLanc.hpp"
#include "internal.cuh"
#include "restart_host.h"

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

// ---- host worker pool ------------------------------------------------------------
// The O(ncv^2) restart math of a batch or a serving lane is one independent
// host routine per problem (a 24-column restart takes ~50 us on one core,
// so 512 problems would hold one core for ~25 ms per cycle).  They run on a
// few worker threads, started on first use and joined at exit; each problem
// writes only its own host mirror, so the result does not depend on which
// thread ran it.  A second caller that finds the pool busy runs its loop
// inline.
class HostPool {
public:
    static HostPool &get() {
        static HostPool pool;
        return pool;
    }
    // fn(i) for i in [0, count); returns when all are done.
    void run(int count, const std::function<void(int)> &fn) {
        std::unique_lock<std::mutex> busy(run_mu_, std::try_to_lock);
        if (count < 4 || !busy.owns_lock() || !start()) {
            for (int i = 0; i < count; ++i) fn(i);
            return;
        }
        {
            std::lock_guard<std::mutex> g(mu_);
            fn_.store(&fn);
            count_.store(count);
            next_.store(0);
            done_ = 0;
            ++gen_;
        }
        cv_.notify_all();
        const int mine = work();
        std::unique_lock<std::mutex> g(mu_);
        done_ += mine;
        done_cv_.wait(g, [&] { return done_ == count_.load(); });
        fn_.store(nullptr);
    }
    ~HostPool() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto &t : threads_) t.join();
    }

private:
    bool start() {
        if (started_) return !threads_.empty();
        started_ = true;
        const unsigned hc = std::thread::hardware_concurrency();
        const int nw = (int)std::min(15u, hc > 1 ? hc - 1 : 0u);
        for (int i = 0; i < nw; ++i) threads_.emplace_back([this] { loop(); });
        return !threads_.empty();
    }
    int work() {
        int n = 0;
        for (int i = next_.fetch_add(1); i < count_.load(); i = next_.fetch_add(1)) {
            (*fn_.load())(i);
            ++n;
        }
        return n;
    }
    void loop() {
        unsigned long long seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> g(mu_);
                cv_.wait(g, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
                if (!fn_.load()) continue;
            }
            const int n = work();
            std::lock_guard<std::mutex> g(mu_);
            done_ += n;
            if (done_ == count_.load()) done_cv_.notify_all();
        }
    }
    std::mutex run_mu_, mu_;
    std::condition_variable cv_, done_cv_;
    std::vector<std::thread> threads_;
    std::atomic<const std::function<void(int)> *> fn_{nullptr};
    std::atomic<int> count_{0}, next_{0};
    int done_ = 0;
    unsigned long long gen_ = 0;
    bool stop_ = false, started_ = false;
};

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
    long long max_row = 0;                      // longest row (entries), general CSR
    int tune[4] = {SPMV_ROWS, SPMV_NNZ, SUBWARP4_MEAN, SUBWARP8_MEAN};   // SpMV unit shape in use
    double tune_us = 0.0, tune_us_default = 0.0;   // measured SpMV time of it / of the default (0: not tuned)
    double sell_us = 0.0;                        // measured SpMV time of the sliced-ELL candidate
    std::vector<SpmvTile> stiles_h;             // entry-balanced SpMV work units (prob = 0)
    SpmvTile *stiles_d = nullptr;
    // sliced-ELL copy (kind 5 units) when the tuner picked it
    long long *sl_ptr_d = nullptr;
    int *sl_len_d = nullptr, *sl_row_d = nullptr, *sl_col_d = nullptr;
    double *sl_val_d = nullptr;
    float *sl_val32_d = nullptr;
    long long sl_elems = 0;
    Sell sell() const { return Sell{sl_ptr_d, sl_len_d, sl_row_d, sl_col_d, sl_val_d, sl_val32_d}; }
    void free_sell() {
        cudaFree(sl_ptr_d); cudaFree(sl_len_d); cudaFree(sl_row_d); cudaFree(sl_col_d);
        cudaFree(sl_val_d); cudaFree(sl_val32_d);
        sl_ptr_d = nullptr; sl_len_d = sl_row_d = sl_col_d = nullptr; sl_val_d = nullptr; sl_val32_d = nullptr;
        sl_elems = 0;
    }
    std::mutex mu;
};

// Split rows into SpMV work units (see SpmvTile): runs of short rows (at most
// prm.rows rows / prm.nnz entries; thread, 4 or 8 lanes per row by the run's
// mean length against prm.sub4 / prm.sub8), runs of up to TPB/16 medium rows,
// and single wide rows.
struct SpmvParams { int rows, nnz, sub4, sub8; };
constexpr SpmvParams SPMV_DEFAULT = {SPMV_ROWS, SPMV_NNZ, SUBWARP4_MEAN, SUBWARP8_MEAN};

static void build_spmv_tiles(const int *rp, int nrows, std::vector<SpmvTile> &out,
                             const SpmvParams &prm = SPMV_DEFAULT) {
    out.clear();
    auto len = [&](int r) { return (long long)rp[r + 1] - rp[r]; };
    int r = 0;
    while (r < nrows) {
        const long long l = len(r);
        if (l > WIDE_ROW) {
            out.push_back({0, r, r + 1, 2});
            ++r;
        } else if (l > LONG_ROW) {
            const int r0 = r;
            while (r < nrows && r - r0 < TPB / 16 && len(r) > LONG_ROW && len(r) <= WIDE_ROW) ++r;
            out.push_back({0, r0, r, 1});
        } else {
            const int r0 = r;
            long long nnz = 0;
            while (r < nrows && r - r0 < prm.rows && len(r) <= LONG_ROW && nnz + len(r) <= prm.nnz) {
                nnz += len(r);
                ++r;
            }
            const long long mean = nnz / (r - r0);
            out.push_back({0, r0, r, mean > prm.sub8 ? 4 : (mean > prm.sub4 ? 3 : 0)});
        }
    }
}

// Sliced-ELL layout of the rows of at most LONG_ROW entries (Sell,
// internal.cuh): windows of SELL_SIGMA consecutive such rows, sorted by
// length (longest first; a counting sort, stable) and cut into slices of
// SELL_C rows.  Longer rows keep their 16-lanes-per-row and CTA-per-row
// units: a lane walking one row of hundreds of entries alone (one dependent
// gather after another) made its warp the kernel's critical path.  Only the slice
// metadata is built here; columns and values are copied on the device.
struct SellBuild {
    std::vector<long long> ptr;
    std::vector<int> len, row;
    std::vector<SpmvTile> units;
    long long elems = 0;
};
static void build_sell(const int *rp, int nrows, SellBuild &B) {
    std::vector<int> win, cnt(LONG_ROW + 2), sorted;
    win.reserve(SELL_SIGMA);
    auto flush = [&]() {
        if (win.empty()) return;
        std::fill(cnt.begin(), cnt.end(), 0);
        for (int r : win) ++cnt[LONG_ROW - (rp[r + 1] - rp[r])];      // longest first
        int acc = 0;
        for (int &c : cnt) { const int t = c; c = acc; acc += t; }
        sorted.assign(win.size(), 0);
        for (int r : win) sorted[cnt[LONG_ROW - (rp[r + 1] - rp[r])]++] = r;
        const int first = (int)B.len.size();
        for (size_t i = 0; i < sorted.size(); i += SELL_C) {
            int mx = 0;
            for (int l = 0; l < SELL_C; ++l) {
                const int r = i + l < sorted.size() ? sorted[i + l] : -1;
                B.row.push_back(r);
                if (r >= 0) mx = std::max(mx, rp[r + 1] - rp[r]);
            }
            B.ptr.push_back(B.elems);
            B.len.push_back(mx);
            B.elems += (long long)mx * SELL_C;
        }
        const int last = (int)B.len.size();
        for (int sl = first; sl < last; sl += SELL_SLICES_PER_UNIT)
            B.units.push_back({0, sl, std::min(last, sl + SELL_SLICES_PER_UNIT), 5});
        win.clear();
    };
    for (int r = 0; r < nrows;) {
        const int l = rp[r + 1] - rp[r];
        if (l > WIDE_ROW) {                     // whole CTA
            B.units.push_back({0, r, r + 1, 2});
            ++r;
        } else if (l > LONG_ROW) {              // runs of medium rows, 16 lanes each
            const int r0 = r;
            while (r < nrows && r - r0 < TPB / 16 && rp[r + 1] - rp[r] > LONG_ROW && rp[r + 1] - rp[r] <= WIDE_ROW) ++r;
            B.units.push_back({0, r0, r, 1});
        } else {
            win.push_back(r);
            ++r;
            if ((int)win.size() == SELL_SIGMA) flush();
        }
    }
    flush();
}

// Device copy of a SellBuild into h (columns and values from h's CSR).
static int upload_sell(hlanc_csr_s *h, const SellBuild &B) {
    cudaStream_t s = h->stream;
    const size_t ns = B.len.size();
    const size_t ne = (size_t)std::max<long long>(B.elems, 1);
    CK(cudaMalloc(&h->sl_ptr_d, sizeof(long long) * std::max<size_t>(ns, 1)));
    CK(cudaMalloc(&h->sl_len_d, sizeof(int) * std::max<size_t>(ns, 1)));
    CK(cudaMalloc(&h->sl_row_d, sizeof(int) * std::max<size_t>(B.row.size(), 1)));
    CK(cudaMalloc(&h->sl_col_d, sizeof(int) * ne));
    CK(cudaMalloc(&h->sl_val_d, sizeof(double) * ne));
    if (h->val32_d) CK(cudaMalloc(&h->sl_val32_d, sizeof(float) * ne));
    h->sl_elems = B.elems;
    if (ns) {
        CK(cudaMemcpyAsync(h->sl_ptr_d, B.ptr.data(), sizeof(long long) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(h->sl_len_d, B.len.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(h->sl_row_d, B.row.data(), sizeof(int) * B.row.size(), cudaMemcpyHostToDevice, s));
        launch_sell_fill(h->rp_d, h->ci_d, h->val_d, (int)ns, h->sl_ptr_d, h->sl_len_d, h->sl_row_d, h->sl_col_d,
                         h->sl_val_d, h->sl_val32_d, s);
        CK(cudaGetLastError());
    }
    return HLANC_OK;
}

// SpMV units tuned per matrix.  The row-length histogram decides whether
// there is anything to choose: when no row has more than SUBWARP4_MEAN
// entries, every short unit runs thread per row whatever the thresholds and
// the default units stand (the Laplacians).  Otherwise a few unit shapes --
// rows per unit and the mean row lengths at which a unit takes 4 / 8 lanes
// per row -- are built and each SpMV is timed on the device (one warm-up,
// best of three, CUDA events), and the fastest is kept.  The sliced-ELL
// layout (build_sell) is one more candidate, kept (a second copy of the
// matrix, with its padding) only when it is the fastest.  Problems of fewer
// than 2^16 rows keep the default: their SpMV is launch-latency bound.
static int autotune_spmv(hlanc_csr_s *h, const int *grp) {
    if (h->nrows < (1 << 16) || h->max_row <= SUBWARP4_MEAN) return HLANC_OK;
    const SpmvParams cand[] = {SPMV_DEFAULT, {256, 4096, SUBWARP4_MEAN, SUBWARP8_MEAN}, {1024, 16384, 6, 16},
                               {1024, 16384, 24, 64}, {1024, 16384, 1 << 30, 1 << 30}};
    const int nc = (int)(sizeof cand / sizeof cand[0]);
    cudaStream_t s = h->stream;
    CK(cudaMemsetAsync(h->xs_d, 0, sizeof(double) * (size_t)std::max(h->ncols, 1), s));
    struct Res {
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        SpmvTile *t = nullptr;
        ~Res() { if (e0) cudaEventDestroy(e0); if (e1) cudaEventDestroy(e1); if (t) cudaFree(t); }
    } r;
    CK(cudaEventCreate(&r.e0));
    CK(cudaEventCreate(&r.e1));
    std::vector<std::vector<SpmvTile>> tiles(nc);
    size_t cap = 0;
    for (int c = 0; c < nc; ++c) {
        build_spmv_tiles(grp, h->nrows, tiles[c], cand[c]);
        cap = std::max(cap, tiles[c].size());
    }
    SellBuild sb;
    build_sell(grp, h->nrows, sb);
    tiles.push_back(sb.units);
    cap = std::max(cap, sb.units.size());
    CK(cudaMalloc(&r.t, sizeof(SpmvTile) * std::max<size_t>(cap, 1)));
    if (int rc = upload_sell(h, sb)) {
        h->free_sell();
        return rc;
    }
    const Sell sl = h->sell();
    int best = 0;
    std::vector<double> us(nc + 1, 0.0);
    for (int c = 0; c <= nc; ++c) {
        const int nt = (int)tiles[c].size();
        if (!nt) continue;
        CK(cudaMemcpyAsync(r.t, tiles[c].data(), sizeof(SpmvTile) * nt, cudaMemcpyHostToDevice, s));
        launch_spmv(h->rp_d, h->ci_d, h->val_d, sl, r.t, nt, h->xs_d, h->ys_d, s);
        float bestms = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
            CK(cudaEventRecord(r.e0, s));
            launch_spmv(h->rp_d, h->ci_d, h->val_d, sl, r.t, nt, h->xs_d, h->ys_d, s);
            CK(cudaEventRecord(r.e1, s));
            CK(cudaEventSynchronize(r.e1));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, r.e0, r.e1));
            bestms = std::min(bestms, ms);
        }
        us[c] = bestms * 1e3;
        if (us[c] < us[best]) best = c;
    }
    h->tune_us_default = us[0];
    h->tune_us = us[best];
    h->sell_us = us[nc];
    if (best == nc) {
        h->tune[0] = -1; h->tune[1] = 0; h->tune[2] = 0; h->tune[3] = 0;
    } else {
        h->tune[0] = cand[best].rows; h->tune[1] = cand[best].nnz; h->tune[2] = cand[best].sub4;
        h->tune[3] = cand[best].sub8;
        CK(cudaStreamSynchronize(s));
        h->free_sell();
    }
    if (best != 0) {
        h->stiles_h.swap(tiles[best]);
        CK(cudaFree(h->stiles_d));
        h->stiles_d = nullptr;
        CK(cudaMalloc(&h->stiles_d, sizeof(SpmvTile) * std::max<size_t>(h->stiles_h.size(), 1)));
        CK(cudaMemcpyAsync(h->stiles_d, h->stiles_h.data(), sizeof(SpmvTile) * h->stiles_h.size(),
                           cudaMemcpyHostToDevice, s));
    }
    CK(cudaStreamSynchronize(s));
    return HLANC_OK;
}

struct hlanc_matrix_s {
    HLanc::dcsr_matrix_t m;
};

namespace hlanc {

// ---- launch profiler ---------------------------------------------------------
struct Profiler {
    std::vector<cudaEvent_t> pool;
    size_t next = 0;
    struct Rec { int cls; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    cudaEvent_t pending = nullptr;
    double host_ms = 0.0;
    long long host_n = 0;
    cudaEvent_t get() {
        if (next == pool.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            pool.push_back(e);
        }
        return pool[next++];
    }
    ~Profiler() {
        for (auto e : pool) cudaEventDestroy(e);
    }
};
static thread_local Profiler *g_prof = nullptr;
static thread_local hlanc_profile_t g_last_prof;
static thread_local bool g_have_prof = false;

void prof_begin(cudaStream_t s) {
    if (!g_prof) return;
    g_prof->pending = g_prof->get();
    cudaEventRecord(g_prof->pending, s);
}
void prof_end(int cls, cudaStream_t s) {
    if (!g_prof || !g_prof->pending) return;
    cudaEvent_t b = g_prof->get();
    cudaEventRecord(b, s);
    g_prof->recs.push_back({cls, g_prof->pending, b});
    g_prof->pending = nullptr;
}

}  // namespace hlanc

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

// Rows per tile: about 4 tiles per SM for large problems (152 SMs), at
// least min_rows (128 for a solo solve), a multiple of 64.
int tile_rows_for(int n, int min_rows = 128) {
    long long tr = ((long long)n + 607) / 608;
    tr = (tr + ROW_ALIGN - 1) / ROW_ALIGN * ROW_ALIGN;
    if (tr < min_rows) tr = min_rows;
    if (tr > (1 << 16)) tr = 1 << 16;
    return (int)tr;
}

// Minimum tile of an engine that runs many problems in one launch: their
// tiles together fill the GPU, so larger tiles cut the per-tile launch and
// reduction work of small problems.  Measured on GB300 against 128 rows: a
// 512-problem batch 1.8x faster at 2048 rows; the 100-request serving mix
// 1.25x faster at 512-1024 rows (slower at 2048: its few resident problems
// need more CTAs each).
constexpr int BATCH_MIN_TILE_ROWS = 2048;
constexpr int SERVE_MIN_TILE_ROWS = 1024;

constexpr int MBOX_STATE = 32;   // doubles reserved for State in a mailbox slot

long long mbox_slot(int m) { return MBOX_STATE + 2LL * m + (long long)m * m + m; }

// ---- one problem's device resources and host mirror --------------------------------
struct ProbRes {
    int n = 0, ncv = 0, nev0 = 0, ld = 0, ntiles = 0, tr = 0, pstride = 0, ngroups = 0;
    int fp32 = 0;
    hlanc_csr_s *csr = nullptr;
    hlanc_host_op_fn host_op = nullptr;
    void *host_ctx = nullptr;
    double *block = nullptr;   // V | r0 | r1 | part | gpart | small
    double *V = nullptr, *r0 = nullptr, *r1 = nullptr, *part = nullptr, *gpart = nullptr, *small = nullptr;
    float *V32 = nullptr;      // FP32 shadow of V (ld x ncv)
    State *st = nullptr;
    unsigned *counter = nullptr;
    double *vout = nullptr;
    int ldo = 0;
    bool own_vout = false;
    size_t bytes = 0;
    int cycles = 0;            // restart cycles launched
    bool live = false;         // resources allocated
    cudaMemPool_t pool = nullptr;        // stream-ordered allocations (serving) when set
    cudaStream_t pool_stream = nullptr;
    // host mirror (host restart)
    std::vector<double> h, ritz_s, bnds_s, Q, values;
    State hs;

    int min_tile_rows = 128;
    static size_t estimate(int n, int ncv, int fp32, int min_rows = 128) {
        const size_t ld = ((size_t)n + ROW_ALIGN - 1) / ROW_ALIGN * ROW_ALIGN;
        const int tr = tile_rows_for(n, min_rows);
        const size_t nt = ((size_t)n + tr - 1) / tr, ng = (nt + RGROUP - 1) / RGROUP;
        const size_t pst = (size_t)((ncv + 2 + 1) & ~1);
        size_t d = ld * ncv + 2 * ld + (nt + ng) * pst + SM_SIZE(ncv);
        size_t b = d * sizeof(double) + 1024 + 4 * ng;
        b += ld * ncv * sizeof(float);    // FP32 shadow of the basis
        b += ld * ncv * sizeof(double);   // Ritz output
        return b;
    }

    cudaError_t dmalloc(void **ptr, size_t b, cudaStream_t s) {
        return pool ? cudaMallocFromPoolAsync(ptr, b, pool, s) : cudaMalloc(ptr, b);
    }
    void dfree(void *ptr) {
        if (!ptr) return;
        if (pool) cudaFreeAsync(ptr, pool_stream);
        else cudaFree(ptr);
    }

    int alloc(cudaStream_t s) {
        pool_stream = s;
        ld = (n + ROW_ALIGN - 1) / ROW_ALIGN * ROW_ALIGN;
        tr = tile_rows_for(n, min_tile_rows);
        ntiles = (n + tr - 1) / tr;
        ngroups = (ntiles + RGROUP - 1) / RGROUP;
        pstride = (ncv + 2 + 1) & ~1;
        const size_t nd = (size_t)ld * ncv + 2 * (size_t)ld + (size_t)(ntiles + ngroups) * pstride + SM_SIZE(ncv);
        bytes = nd * sizeof(double);
        CK(dmalloc((void **)&block, bytes, s));
        live = true;
        CK(cudaMemsetAsync(block, 0, bytes, s));
        V = block;
        r0 = V + (size_t)ld * ncv;
        r1 = r0 + ld;
        part = r1 + ld;
        gpart = part + (size_t)ntiles * pstride;
        small = gpart + (size_t)ngroups * pstride;
        const size_t sb = 512 + 4 * ((size_t)ngroups + 1);
        void *sp = nullptr;
        CK(dmalloc(&sp, sb, s));
        CK(cudaMemsetAsync(sp, 0, sb, s));
        st = (State *)sp;
        counter = (unsigned *)((char *)sp + 512);
        bytes += sb;
        CK(dmalloc((void **)&V32, (size_t)ld * ncv * sizeof(float), s));
        CK(cudaMemsetAsync(V32, 0, (size_t)ld * ncv * sizeof(float), s));
        bytes += (size_t)ld * ncv * sizeof(float);
        h.assign(2 * ncv, 0.0);
        ritz_s.assign(ncv, 0.0);
        bnds_s.assign(ncv, 0.0);
        Q.assign((size_t)ncv * ncv, 0.0);
        values.assign(ncv, 0.0);
        return HLANC_OK;
    }
    // Ritz-vector output owned by the problem (ld x ncv)
    int alloc_vout(cudaStream_t s) {
        CK(dmalloc((void **)&vout, sizeof(double) * (size_t)ld * ncv, s));
        own_vout = true;
        ldo = ld;
        return HLANC_OK;
    }
    void release() {
        dfree(block);
        dfree(st);
        dfree(V32);
        if (own_vout) dfree(vout);
        block = nullptr; st = nullptr; V32 = nullptr; vout = nullptr; own_vout = false;
        live = false;
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
    S.wait_limit = o.wait_limit;
    return S;
}

// ---- the engine: a set of problems sharing launches ------------------------------
class Engine {
public:
    int dev = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool use_graphs = true;
    bool device_restart = false;
    cudaMemPool_t pool = nullptr;        // when set, problems allocate from it on `stream`
    int min_tile_rows = 128;
    bool basis_tc = true;                // basis update on the tensor cores when the shape fits
    int cgs_mode = HLANC_CGS_AUTO;       // CGS panels split between the FP64 and the integer pipes
    int cycle_mode = HLANC_CYCLE_AUTO;   // whole extensions in one cooperative launch when eligible
    // one-launch extensions (kernels_cycle.cu): CTA table, barrier counters
    CycTileH *C_d = nullptr;
    unsigned *bars_d = nullptr;
    double *xpart_d = nullptr;           // nctas_cap x 3 (MAXNCV + 2) partial sums
    int nctas = 0, nctas_cap = 0;
    long long rows_active = 0;           // rows of all problems in the launch tables
    Problem one_h;                       // descriptor of a single-problem launch table
    int one_tr = 0;                      // its tile rows (0: several problems)
    const Problem *one() const { return one_tr > 0 ? &one_h : nullptr; }
    std::vector<ProbRes> probs;
    std::vector<int> active;             // problems in the launch tables, in slot order
    Problem *P_d = nullptr;
    Tile *T_d = nullptr;
    SpmvTile *S_d = nullptr;             // entry-balanced SpMV units of all active problems
    int ntiles = 0, nslots_cap = 0, ntiles_cap = 0, nstiles = 0, nstiles_cap = 0;
    int max_ncv = 0;
    bool fp32_any = false;
    // A captured cycle and the kernels it holds (total and per counted
    // variant), added to the launch counters on every replay.
    struct Captured {
        cudaGraphExec_t exec = nullptr;
        long long kernels = 0;
        long long variants[HLANC_KL_KINDS] = {};
    };
    std::map<long long, Captured> graphs;
    // host-restart mailbox
    std::vector<long long> off_h;
    long long *off_d = nullptr;
    int *flag_d = nullptr, *flag_h = nullptr;
    double *mbox_d = nullptr, *mbox_h = nullptr;
    long long mbox_used = 0, mbox_cap = 0;
    int flags_cap = 0;
    // host-operator staging
    double *xs_h = nullptr, *ys_h = nullptr, *xs_d = nullptr;
    size_t xs_cap = 0;

    ~Engine() {
        DevGuard g(dev);
        drop_graphs();
        for (auto &p : probs) p.release();
        if (P_d) cudaFree(P_d);
        if (T_d) cudaFree(T_d);
        if (S_d) cudaFree(S_d);
        if (C_d) cudaFree(C_d);
        if (bars_d) cudaFree(bars_d);
        if (xpart_d) cudaFree(xpart_d);
        if (off_d) cudaFree(off_d);
        if (flag_d) cudaFree(flag_d);
        if (mbox_d) cudaFree(mbox_d);
        if (mbox_h) cudaFreeHost(mbox_h);
        if (flag_h) cudaFreeHost(flag_h);
        if (xs_h) cudaFreeHost(xs_h);
        if (ys_h) cudaFreeHost(ys_h);
        if (xs_d) cudaFree(xs_d);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }

    int init(int device, void *user_stream, bool graphs_on, bool dev_restart) {
        dev = device;
        use_graphs = graphs_on;
        device_restart = dev_restart;
        if (user_stream) {
            stream = (cudaStream_t)user_stream;
        } else {
            CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
            own_stream = true;
        }
        return HLANC_OK;
    }

    void drop_graphs() {
        for (auto &kv : graphs) cudaGraphExecDestroy(kv.second.exec);
        graphs.clear();
    }

    int add(int n, int nev, int ncv, hlanc_csr_s *csr, hlanc_host_op_fn host_op, void *host_ctx, int fp32,
            const hlanc_opts_t &o, int *index) {
        ProbRes p;
        p.n = n; p.ncv = ncv; p.nev0 = nev; p.csr = csr; p.host_op = host_op; p.host_ctx = host_ctx;
        p.fp32 = fp32;
        p.pool = pool;
        p.min_tile_rows = min_tile_rows;
        int rc = p.alloc(stream);
        if (rc) { p.release(); return rc == HLANC_ERR_CUDA ? HLANC_ERR_ALLOC : rc; }
        State S = initial_state(nev, ncv, o);
        p.hs = S;
        CK(cudaMemcpyAsync(p.st, &S, sizeof S, cudaMemcpyHostToDevice, stream));
        probs.push_back(std::move(p));
        *index = (int)probs.size() - 1;
        return HLANC_OK;
    }

    // The hybrid CGS kernels pay a little latency per launch (the scale scan
    // of w, per-row conversions) for throughput; launches over few rows are
    // latency-bound and keep the FP64 kernels (measured on GB300: the
    // 10,000-row Laplacian solve took 100.6 ms hybrid against 90.1 ms FP64;
    // the 4.1M-row solve 4.95 s against 5.41 s).
    static constexpr long long CGS_HYBRID_MIN_ROWS = 1 << 18;
    int cgs_flags() const {
        const bool hy = cgs_mode == HLANC_CGS_HYBRID || (cgs_mode == HLANC_CGS_AUTO && rows_active >= CGS_HYBRID_MIN_ROWS);
        return (hy ? CGS_PROJ_HYBRID : 0) | (cgs_mode != HLANC_CGS_FP64 ? CGS_APPLY_SHADOW : 0);
    }

    // Problems whose whole extension runs in one cooperative launch: every
    // active problem has a device operator with rows of at most LONG_ROW
    // entries (thread-per-row SpMV), and together they have few enough rows
    // that the per-phase launches are latency-bound.  Each problem gets a
    // group of CTAs of about cycle_rows_per_cta() rows, no more than its
    // reduction slots (tiles), and the groups together fit the co-resident
    // capacity.  Measured on GB300 (whole solves, one launch per extension
    // against per-phase launches): 2-D Laplacian 10,000 rows 61.7 vs 93.7 ms,
    // banded 20,000 rows 14.0 vs 24.9 ms, 3-D Laplacian 27,000 rows 60.4 vs
    // 65.6 ms, but 125,000 rows 204 vs 151 ms; a power-law graph of 16,384
    // rows (rows up to ~700 entries, one thread each) 91.6 vs 60.8 ms.
    static constexpr long long CYCLE_MAX_ROWS = 48 * 1024;
    int rc_cycle = 0;
    int plan_cycle() {
        nctas = 0;
        if (cycle_mode == HLANC_CYCLE_OFF || active.empty() || rows_active > CYCLE_MAX_ROWS) return HLANC_OK;
        for (int pi : active) {
            const ProbRes &p = probs[pi];
            if (!p.csr || p.csr->max_row > LONG_ROW) return HLANC_OK;
        }
        static int cap_dev[64] = {0};
        int d = 0;
        cudaGetDevice(&d);
        int cap = (d < 64 && cap_dev[d]) ? cap_dev[d] : cycle_capacity();
        if (d < 64) cap_dev[d] = cap;
        if (cap <= 0) return HLANC_OK;
        const long long per = cycle_rows_per_cta();
        std::vector<CycTileH> C;
        for (size_t a = 0; a < active.size(); ++a) {
            const ProbRes &p = probs[active[a]];
            int nb = (int)std::min<long long>((p.n + per - 1) / per, p.ntiles);
            nb = std::max(nb, 1);
            const int rows = (p.n + nb - 1) / nb;
            for (int r = 0; r < nb; ++r)
                C.push_back({(int)a, r, nb, r * rows, std::min(p.n, (r + 1) * rows), 0});
        }
        if ((long long)C.size() > cap) return HLANC_OK;
        if ((int)C.size() > nctas_cap || !C_d) {
            if (C_d) cudaFree(C_d);
            nctas_cap = (int)C.size() + 64;
            CK(cudaMalloc(&C_d, sizeof(CycTileH) * nctas_cap));
            if (xpart_d) cudaFree(xpart_d);
            xpart_d = nullptr;
            CK(cudaMalloc(&xpart_d, sizeof(double) * 3 * (MAXNCV + 2) * (size_t)nctas_cap));
        }
        if (!bars_d || nslots_cap > bars_cap) {
            if (bars_d) cudaFree(bars_d);
            bars_cap = nslots_cap;
            CK(cudaMalloc(&bars_d, sizeof(unsigned) * bars_cap));
        }
        CK(cudaMemcpyAsync(C_d, C.data(), sizeof(CycTileH) * C.size(), cudaMemcpyHostToDevice, stream));
        nctas = (int)C.size();
        return HLANC_OK;
    }
    int bars_cap = 0;

    // The steps of one extension: one cooperative launch, or the per-phase
    // launches of launch_step.
    void enqueue_steps(int steps) {
        if (nctas > 0) {
            (void)launch_cycle(P_d, C_d, nctas, bars_d, xpart_d, (int)active.size(), steps, stream);
            return;
        }
        for (int s = 0; s < steps; ++s)
            launch_step(P_d, T_d, ntiles, S_d, nstiles, s, fp32_any, false, cgs_flags(), one(), one_tr, stream);
    }

    // Rebuild the descriptor/tile tables and the mailbox layout for `active`.
    int upload() {
        std::vector<Problem> P(active.size());
        std::vector<Tile> T;
        std::vector<SpmvTile> ST;
        max_ncv = 0;
        fp32_any = false;
        rows_active = 0;
        off_h.assign(active.size(), 0);
        long long off = 0;
        for (size_t a = 0; a < active.size(); ++a) {
            ProbRes &p = probs[active[a]];
            Problem &q = P[a];
            memset(&q, 0, sizeof q);
            if (p.csr) {
                q.row_ptr = p.csr->rp_d; q.col = p.csr->ci_d; q.val = p.csr->val_d;
                q.val32 = p.fp32 ? p.csr->val32_d : nullptr;
                q.sell = p.csr->sell();
            }
            q.n = p.n; q.ld = p.ld; q.ncv = p.ncv; q.nev0 = p.nev0;
            q.tile0 = (int)T.size(); q.ntiles = p.ntiles;
            q.fp32 = p.fp32; q.pstride = p.pstride;
            q.V = p.V; q.V32 = p.V32; q.r0 = p.r0; q.r1 = p.r1; q.part = p.part; q.gpart = p.gpart; q.counter = p.counter;
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
            if (p.csr)
                for (SpmvTile st : p.csr->stiles_h) {
                    st.prob = (int)a;
                    ST.push_back(st);
                }
            max_ncv = std::max(max_ncv, p.ncv);
            fp32_any = fp32_any || p.fp32;
            rows_active += p.n;
            off_h[a] = off;
            off += mbox_slot(p.ncv);
        }
        mbox_used = off;
        const int na = std::max<int>((int)active.size(), 1);
        if (na > nslots_cap) {
            if (P_d) cudaFree(P_d);
            if (off_d) cudaFree(off_d);
            if (flag_d) cudaFree(flag_d);
            if (flag_h) cudaFreeHost(flag_h);
            nslots_cap = na + 8;
            CK(cudaMalloc(&P_d, sizeof(Problem) * nslots_cap));
            CK(cudaMalloc(&off_d, sizeof(long long) * nslots_cap));
            CK(cudaMalloc(&flag_d, sizeof(int) * nslots_cap));
            CK(cudaMallocHost(&flag_h, sizeof(int) * nslots_cap));
        }
        if ((int)T.size() > ntiles_cap || !T_d) {
            if (T_d) cudaFree(T_d);
            ntiles_cap = std::max<int>((int)T.size(), 1) + 64;
            CK(cudaMalloc(&T_d, sizeof(Tile) * ntiles_cap));
        }
        if (mbox_used > mbox_cap) {
            if (mbox_d) cudaFree(mbox_d);
            if (mbox_h) cudaFreeHost(mbox_h);
            mbox_cap = mbox_used + 4096;
            CK(cudaMalloc(&mbox_d, sizeof(double) * mbox_cap));
            CK(cudaMallocHost(&mbox_h, sizeof(double) * mbox_cap));
        }
        if ((int)ST.size() > nstiles_cap || !S_d) {
            if (S_d) cudaFree(S_d);
            nstiles_cap = std::max<int>((int)ST.size(), 1) + 64;
            CK(cudaMalloc(&S_d, sizeof(SpmvTile) * nstiles_cap));
        }
        nstiles = (int)ST.size();
        if (!ST.empty()) CK(cudaMemcpyAsync(S_d, ST.data(), sizeof(SpmvTile) * ST.size(), cudaMemcpyHostToDevice, stream));
        if ((rc_cycle = plan_cycle())) return rc_cycle;
        ntiles = (int)T.size();
        one_tr = 0;
        if (active.size() == 1) {
            one_h = P[0];
            one_tr = probs[active[0]].tr;
        }
        if (!P.empty()) CK(cudaMemcpyAsync(P_d, P.data(), sizeof(Problem) * P.size(), cudaMemcpyHostToDevice, stream));
        if (!T.empty()) CK(cudaMemcpyAsync(T_d, T.data(), sizeof(Tile) * T.size(), cudaMemcpyHostToDevice, stream));
        if (!active.empty())
            CK(cudaMemcpyAsync(off_d, off_h.data(), sizeof(long long) * active.size(), cudaMemcpyHostToDevice, stream));
        for (size_t a = 0; a < active.size(); ++a) flag_h[a] = 0;
        CK(cudaStreamSynchronize(stream));   // off_h / flag_h are reused by later async copies
        drop_graphs();
        return HLANC_OK;
    }

    // A bounded device wait that gave up leaves State::err set; the host
    // reads it with the State after every cycle and abandons the solve.
    int device_error() const {
        for (int p : active)
            if (probs[p].hs.err != DEV_ERR_NONE) return HLANC_ERR_DEVICE_TIMEOUT;
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
            CK(cudaStreamSynchronize(stream));   // o.start may be pageable / short-lived
        } else {
            launch_start_vector(P_d, T_d, ntiles, slot_of(prob), o.seed, stream);
        }
        return HLANC_OK;
    }

    int norm_init() {
        launch_norm_init(P_d, T_d, ntiles, stream);
        CK(cudaGetLastError());
        return HLANC_OK;
    }

    // graph key for the basis kernel instantiation launch_basis picks
    // Width class of the basis update for an (adjusted) nev: the tensor-core
    // kernel takes nev + 1 <= 64 outputs (nev <= 63, bucket 63), the FP64
    // kernel up to 64 outputs in registers, and the wide kernel the rest
    // (ncv > 64 only).
    static int basis_bucket(int nev) {
        if (nev <= 0) return 0;
        const int q = (nev + 3) / 4;
        return q <= 10 ? 4 * q : q <= 12 ? 48 : q <= 14 ? 56 : nev <= 63 ? 63 : nev == 64 ? 64 : HLANC_MAX_NCV;
    }

    // Device part of one cycle: apply pending restarts, extend, (restart), gather.
    void enqueue_cycle(int steps, int basis_nev) {
        const int na = (int)active.size();
        if (!device_restart) launch_scatter(P_d, na, off_d, flag_d, mbox_d, stream);
        if (basis_nev > 0) launch_basis(P_d, T_d, ntiles, max_ncv, basis_bucket(basis_nev), basis_tc, stream);
        enqueue_steps(steps);
        if (device_restart) launch_restart(P_d, na, max_ncv, stream);
        launch_gather(P_d, na, off_d, mbox_d, stream);
    }

    int push_mailbox() {
        const int na = (int)active.size();
        CK(cudaMemcpyAsync(flag_d, flag_h, sizeof(int) * na, cudaMemcpyHostToDevice, stream));
        bool any = false;
        for (int a = 0; a < na; ++a) any = any || flag_h[a];
        if (any) CK(cudaMemcpyAsync(mbox_d, mbox_h, sizeof(double) * mbox_used, cudaMemcpyHostToDevice, stream));
        return HLANC_OK;
    }

    // Copy the gathered State/h of the active problems into their host
    // mirrors; with `only`, just those problems (a finalisation must not
    // overwrite the restart decisions of problems still running).
    int pull_mailbox(const std::vector<int> *only = nullptr) {
        int rc = pull_async();
        if (rc) return rc;
        CK(cudaStreamSynchronize(stream));
        CK(cudaGetLastError());
        unpack_mailbox(only);
        return HLANC_OK;
    }
    // Device mailbox -> pinned host copy, ordered after the cycle on `stream`.
    int pull_async() {
        CK(cudaMemcpyAsync(mbox_h, mbox_d, sizeof(double) * mbox_used, cudaMemcpyDeviceToHost, stream));
        return HLANC_OK;
    }
    // Host copy of the mailbox -> the problems' State/h mirrors.
    void unpack_mailbox(const std::vector<int> *only = nullptr) {
        for (size_t a = 0; a < active.size(); ++a) {
            if (only && std::find(only->begin(), only->end(), active[a]) == only->end()) continue;
            ProbRes &p = probs[active[a]];
            const double *slot = mbox_h + off_h[a];
            memcpy(&p.hs, slot, sizeof(State));
            if (!device_restart) memcpy(p.h.data(), slot + MBOX_STATE, sizeof(double) * 2 * p.ncv);
        }
    }

    // One restart cycle of every active device-operator problem.
    int run_cycle(int steps, int basis_nev) {
        int rc = push_mailbox();
        if (rc) return rc;
        const bool graphs_now = use_graphs && !g_prof;
        if (!graphs_now) {
            enqueue_cycle(steps, basis_nev);
            CK(cudaGetLastError());
        } else {
            const long long key = (long long)steps * 1024 + basis_bucket(basis_nev);
            auto it = graphs.find(key);
            if (it == graphs.end()) {
                // the enqueue counts the captured kernels once, for this
                // first replay
                Captured c;
                long long v0[HLANC_KL_KINDS];
                for (int k = 0; k < HLANC_KL_KINDS; ++k) v0[k] = variant_counter(k).load();
                const long long k0 = launch_counter().load();
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                enqueue_cycle(steps, basis_nev);
                CK(cudaStreamEndCapture(stream, &g));
                c.kernels = launch_counter().load() - k0;
                for (int k = 0; k < HLANC_KL_KINDS; ++k) c.variants[k] = variant_counter(k).load() - v0[k];
                cudaError_t e = cudaGraphInstantiate(&c.exec, g, 0);
                cudaGraphDestroy(g);
                CK(e);
                it = graphs.emplace(key, c).first;
            } else {
                launch_counter() += it->second.kernels;
                for (int k = 1; k < HLANC_KL_KINDS; ++k) variant_counter(k) += it->second.variants[k];
            }
            CK(cudaGraphLaunch(it->second.exec, stream));
        }
        for (size_t a = 0; a < active.size(); ++a) probs[active[a]].cycles += 1;
        return pull_mailbox();
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
        int rc = push_mailbox();
        if (rc) return rc;
        const int na = (int)active.size();
        if (!device_restart) launch_scatter(P_d, na, off_d, flag_d, mbox_d, stream);
        if (basis_nev > 0) launch_basis(P_d, T_d, ntiles, max_ncv, basis_bucket(basis_nev), basis_tc, stream);
        const int k = p.hs.k;
        for (int s = 0; s < steps; ++s) {
            const int j = k + s;
            launch_prep_ext(P_d, T_d, ntiles, s, xs_d, stream);
            CK(cudaMemcpyAsync(xs_h, xs_d, sizeof(double) * p.n, cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            if (p.host_op(p.host_ctx, xs_h, ys_h) != 0) return HLANC_ERR_CALLBACK;
            double *w = ((j + 1) & 1) ? p.r1 : p.r0;
            CK(cudaMemcpyAsync(w, ys_h, sizeof(double) * p.n, cudaMemcpyHostToDevice, stream));
            launch_step(P_d, T_d, ntiles, S_d, nstiles, s, false, true, cgs_flags(), one(), one_tr, stream);
        }
        if (device_restart) launch_restart(P_d, na, max_ncv, stream);
        launch_gather(P_d, na, off_d, mbox_d, stream);
        CK(cudaGetLastError());
        p.cycles += 1;
        return pull_mailbox();
    }

    // Host restart of every problem whose extension just finished.  Fills the
    // mailbox for the next cycle; returns the number still running, the
    // largest nev to apply and the largest np.
    void host_restarts(int *running, int *nev_max, int *np_max) {
        *running = 0; *nev_max = 0; *np_max = 0;
        const double t0 = now_s();
        // the problems due for a restart, computed on the host pool
        std::vector<int> due;
        std::vector<host::RestartIO> ios;
        std::vector<int> rss;
        if (!device_restart) {
            for (size_t a = 0; a < active.size(); ++a) {
                const ProbRes &p = probs[active[a]];
                const State &S = p.hs;
                if (S.status != ST_RUNNING || S.phase != PH_EXTEND || S.iter < 0) continue;
                host::RestartIO io;
                io.ncv = p.ncv; io.nev0 = S.nev0; io.np0 = S.np0; io.max_iter = S.max_iter;
                io.tol = S.tol; io.eps23 = S.eps23; io.rnorm = S.rnorm; io.iter = S.iter;
                io.h = probs[active[a]].h.data(); io.ritz_s = probs[active[a]].ritz_s.data();
                io.bnds_s = probs[active[a]].bnds_s.data(); io.Q = probs[active[a]].Q.data();
                due.push_back((int)a);
                ios.push_back(io);
            }
            rss.assign(due.size(), 0);
            HostPool::get().run((int)due.size(), [&](int i) { rss[i] = host::restart(ios[i]); });
        }
        size_t q = 0;
        for (size_t a = 0; a < active.size(); ++a) {
            ProbRes &p = probs[active[a]];
            flag_h[a] = 0;
            State &S = p.hs;
            if (device_restart) {
                if (S.status == ST_RUNNING && S.phase == PH_APPLY) {
                    ++*running;
                    *nev_max = std::max(*nev_max, S.nev);
                    *np_max = std::max(*np_max, S.np);
                }
                continue;
            }
            if (q >= due.size() || due[q] != (int)a) continue;
            const host::RestartIO &io = ios[q];
            const int rs = rss[q];
            ++q;
            S.iter = io.iter;
            S.nconv = io.nconv;
            double *slot = mbox_h + off_h[a];
            if (rs == host::RS_APPLY) {
                S.nev = io.nev; S.np = io.np; S.k = io.nev; S.phase = PH_APPLY;
                memcpy(slot + MBOX_STATE, p.h.data(), sizeof(double) * 2 * p.ncv);
                memcpy(slot + MBOX_STATE + 2 * p.ncv, p.Q.data(), sizeof(double) * p.ncv * p.ncv);
                flag_h[a] = 1;
                ++*running;
                *nev_max = std::max(*nev_max, S.nev);
                *np_max = std::max(*np_max, S.np);
            } else {
                S.status = rs == host::RS_CONVERGED ? ST_CONVERGED
                         : rs == host::RS_FAILED ? ST_FAILED : ST_NOT_CONVERGED;
                S.phase = PH_DONE;
                flag_h[a] = 2;
            }
            memcpy(slot, &S, sizeof(State));
        }
        if (g_prof) {
            g_prof->host_ms += (now_s() - t0) * 1e3;
            g_prof->host_n += 1;
        }
    }

    // Converged problems -> values and Ritz vectors (into each p.vout, ldo).
    int finalize_many(const std::vector<int> &which) {
        for (int prob : which) {
            ProbRes &p = probs[prob];
            if (!p.vout) {
                CK(cudaMalloc(&p.vout, sizeof(double) * (size_t)p.ld * p.ncv));
                p.own_vout = true;
                p.ldo = p.ld;
            }
        }
        int rc = upload();     // descriptors carry vout/ldo
        if (rc) return rc;
        if (device_restart) {
            launch_finalize(P_d, (int)active.size(), max_ncv, stream);
        } else {
            for (size_t q = 0; q < active.size(); ++q) flag_h[q] = 0;
            std::vector<int> conv;
            for (int prob : which)
                if (probs[prob].hs.status == ST_CONVERGED) conv.push_back(prob);
            std::vector<int> frc(conv.size(), 0);
            HostPool::get().run((int)conv.size(), [&](int i) {
                ProbRes &p = probs[conv[i]];
                const State &S = p.hs;
                host::FinalizeIO io;
                io.ncv = p.ncv; io.nev0 = S.nev0; io.np0 = S.np0; io.nconv = S.nconv;
                io.tol = S.tol; io.eps23 = S.eps23;
                io.h = p.h.data(); io.ritz_s = p.ritz_s.data(); io.bnds_s = p.bnds_s.data();
                io.values = p.values.data();
                io.Q2 = mbox_h + off_h[slot_of(conv[i])] + MBOX_STATE + 2 * p.ncv;
                frc[i] = host::finalize(io);
            });
            for (size_t i = 0; i < conv.size(); ++i) {
                ProbRes &p = probs[conv[i]];
                const int a = slot_of(conv[i]);
                State &S = p.hs;
                double *slot = mbox_h + off_h[a];
                if (frc[i]) {
                    S.status = ST_FAILED;
                    S.fin = 2;
                    flag_h[a] = 2;
                } else {
                    memcpy(slot + MBOX_STATE + 2 * p.ncv + (size_t)p.ncv * p.ncv, p.values.data(),
                           sizeof(double) * p.ncv);
                    S.fin = 1;
                    flag_h[a] = 3;
                }
                memcpy(slot, &S, sizeof(State));
            }
            if ((rc = push_mailbox())) return rc;
            launch_scatter(P_d, (int)active.size(), off_d, flag_d, mbox_d, stream);
        }
        launch_ritz(P_d, T_d, ntiles, max_ncv, basis_tc, stream);
        launch_gather(P_d, (int)active.size(), off_d, mbox_d, stream);
        CK(cudaGetLastError());
        for (size_t q = 0; q < active.size(); ++q) flag_h[q] = 0;
        if ((rc = pull_mailbox(&which))) return rc;
        for (int pi : which)   // a bounded tensor-core wait of the Ritz kernel that gave up
            if (probs[pi].hs.err != DEV_ERR_NONE) return HLANC_ERR_DEVICE_TIMEOUT;
        return HLANC_OK;
    }
    int finalize(int prob) { return finalize_many(std::vector<int>{prob}); }

    // Release a finished problem's device memory (serving).
    void retire(int prob) {
        probs[prob].release();
        std::vector<double>().swap(probs[prob].Q);
    }
};

// Run every problem in E.active to a terminal state.
int drive(Engine &E) {
    int steps = 0, np0max = 0;
    bool host_path = false;
    for (int p : E.active) {
        steps = std::max(steps, E.probs[p].ncv);
        np0max = std::max(np0max, E.probs[p].ncv - E.probs[p].nev0);
        host_path = host_path || !E.probs[p].csr;
    }
    int basis_nev = 0;
    for (;;) {
        int rc = host_path ? E.run_cycle_host(E.active[0], steps, basis_nev) : E.run_cycle(steps, basis_nev);
        if (rc) return rc;
        if ((rc = E.device_error())) return rc;
        int running, nev_max, np_max;
        E.host_restarts(&running, &nev_max, &np_max);
        if (!running) break;
        basis_nev = nev_max;
        // later cycles launch the largest possible extension (np0 steps);
        // steps beyond a problem's current np exit at once on the device, so
        // one captured graph serves every cycle
        steps = host_path ? np_max : np0max;
    }
    // push terminal states to the device
    int rc = E.push_mailbox();
    if (rc) return rc;
    if (!E.device_restart) launch_scatter(E.P_d, (int)E.active.size(), E.off_d, E.flag_d, E.mbox_d, E.stream);
    for (size_t a = 0; a < E.active.size(); ++a) E.flag_h[a] = 0;
    CK(cudaStreamSynchronize(E.stream));
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
    // projection 8 n c + 8 n; update 8 n (c - t) + 4 n t + 16 n (t columns from the FP32 copy)
    stats->bytes_cgs = 16.0 * n * (double)S.sumc - 4.0 * n * (double)S.sumt + 24.0 * n * (double)S.passes;
    stats->bytes_restart = (8.0 * n * p.ncv + 16.0 * n) * S.napply + 12.0 * n * (double)S.sumnev;
    stats->cgs_update_fp32_share = S.sumc > 0 ? (double)S.sumt / (double)S.sumc : 0.0;
    stats->refine_residual = -1.0;
}

void fill_profile(const State &S, const ProbRes &p, double nnz, int fp32) {
    if (!g_prof) return;
    hlanc_profile_t &P = g_last_prof;
    memset(&P, 0, sizeof P);
    cudaDeviceSynchronize();
    for (auto &r : g_prof->recs) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.a, r.b);
        P.launches[r.cls] += 1;
        P.ms[r.cls] += ms;
    }
    const double n = p.n, m = p.ncv;
    P.bytes[KC_SPMV] = (fp32 ? (8.0 * nnz + 4.0 * (n + 1) + 24.0 * n) : (12.0 * nnz + 4.0 * (n + 1) + 32.0 * n)) * S.spmv;
    P.flops[KC_SPMV] = 2.0 * nnz * S.spmv;
    P.bytes[KC_PROJ] = 8.0 * n * S.sumc + 8.0 * n * S.passes;
    P.flops[KC_PROJ] = 2.0 * n * S.sumc;
    P.bytes[KC_APPLY] = 8.0 * n * (S.sumc - S.sumt) + 4.0 * n * S.sumt + 16.0 * n * S.passes;
    P.flops[KC_APPLY] = 2.0 * n * S.sumc + 2.0 * n * S.passes;
    P.bytes[KC_BASIS] = (8.0 * n * m + 16.0 * n) * S.napply + 12.0 * n * S.sumnev;   // V, FP32 copy
    P.flops[KC_BASIS] = 2.0 * n * m * (S.sumnev + S.napply);
    P.bytes[KC_RITZ] = 16.0 * n * m;
    P.flops[KC_RITZ] = 2.0 * n * m * m;
    P.launches[KC_HOST] = g_prof->host_n;
    P.ms[KC_HOST] = g_prof->host_ms;
    if (P.launches[KC_CYCLE] > 0) {     // the extensions ran as one launch each: their bytes are class 7's
        for (int c : {KC_SPMV, KC_PROJ, KC_APPLY}) {
            if (P.launches[c] > 0) continue;
            P.bytes[KC_CYCLE] += P.bytes[c];
            P.flops[KC_CYCLE] += P.flops[c];
            P.bytes[c] = P.flops[c] = 0.0;
        }
    }
    g_have_prof = true;
}

__global__ void k_sum_columns(const double *__restrict__ Y, int ld, int n, int k, double *__restrict__ out) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < k; ++i) s += Y[(size_t)i * ld + r];
        out[r] = s;
    }
}

int map_status(int st) { return st == ST_CONVERGED ? HLANC_OK : HLANC_NOT_CONVERGED; }

// Column-by-column copy through the device's address space (blockIdx.y =
// column, w elements of T per column).
template <typename T>
__global__ void __launch_bounds__(256) k_copy_cols(const T *__restrict__ src, size_t sp, T *__restrict__ dst,
                                                   size_t dp, size_t w) {
    const T *c = src + (size_t)blockIdx.y * sp;
    T *d = dst + (size_t)blockIdx.y * dp;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < w; i += (size_t)gridDim.x * blockDim.x)
        d[i] = c[i];
}

// Device -> host copy of `height` columns of `width` bytes, synchronous.
//  - A large pinned destination that is mapped into this device's address
//    space is written by a copy kernel.  Measured on this machine's GB300
//    machines (1.97 GB of Ritz vectors): the DMA copy took 10 ms on a quiet
//    host but 130-230 ms inside some solver processes, where stores from
//    the SMs into the same kind of buffer took 34 ms; on a quiet host the
//    kernel copy takes 10 ms like the DMA.
//  - A large pageable destination (the reference API's `new double[]`) is
//    page-locked for the copy, so it runs as one DMA instead of a staged
//    pageable copy (2 GB of Ritz vectors in 1.65 s staged).
int copy_d2h_2d(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t height,
                cudaStream_t s) {
    const size_t span = height ? dpitch * (height - 1) + width : 0;
    bool registered = false;
    if (span >= ((size_t)64 << 20)) {
        cudaPointerAttributes a;
        int dev = -1;
        cudaGetDevice(&dev);
        if (cudaPointerGetAttributes(&a, dst) == cudaSuccess) {
            const uintptr_t dp = (uintptr_t)a.devicePointer, sp = (uintptr_t)src;
            if (a.type == cudaMemoryTypeHost && dp && a.device == dev && height <= 65535 &&
                ((width | dpitch | spitch | dp | sp) & 7) == 0) {
                const unsigned gx = (unsigned)std::max<size_t>(1, (size_t)1216 / height);
                const dim3 grid(gx, (unsigned)height);
                if (((width | dpitch | spitch | dp | sp) & 15) == 0)
                    k_copy_cols<double2><<<grid, 256, 0, s>>>(static_cast<const double2 *>(src), spitch / 16,
                                                              reinterpret_cast<double2 *>(dp), dpitch / 16,
                                                              width / 16);
                else
                    k_copy_cols<double><<<grid, 256, 0, s>>>(static_cast<const double *>(src), spitch / 8,
                                                             reinterpret_cast<double *>(dp), dpitch / 8, width / 8);
                launch_counter() += 1;
                cudaError_t e = cudaGetLastError();
                if (e == cudaSuccess) e = cudaStreamSynchronize(s);
                CK(e);
                return HLANC_OK;
            }
            if (a.type == cudaMemoryTypeUnregistered)
                registered = cudaHostRegister(dst, span, cudaHostRegisterDefault) == cudaSuccess;
        }
        cudaGetLastError();   // an unregistrable range only means the staged copy
    }
    cudaError_t e = cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (registered) cudaHostUnregister(dst);
    CK(e);
    return HLANC_OK;
}

// Mixed precision: the FP32-SpMV phase stops at a relative tolerance of
// 1e-6 (FP32 rounding of the SpMV sits near 1e-7) and gets a quarter of the
// restart budget; the FP64 phase then has the whole budget.
hlanc_opts_t fp32_phase_opts(const hlanc_opts_t &o) {
    hlanc_opts_t o1 = o;
    o1.tol = std::max(o.tol > 0 ? o.tol : 0.0, 1e-6);
    const int mr = o.max_restarts > 0 ? o.max_restarts : 200;
    o1.max_restarts = std::max(1, mr / 4);
    return o1;
}

// Start vector of the FP64 phase, written into r0: the sum of the FP32
// phase's (refined) Ritz vectors when it converged (they are in vout), else
// that phase's current first Lanczos vector V[:, 0] -- the start vector its
// restarts have filtered so far.
void fp64_phase_start(const ProbRes &p, cudaStream_t s) {
    if (p.hs.status == ST_CONVERGED && p.hs.fin == 2)
        k_sum_columns<<<304, 256, 0, s>>>(p.vout, p.ldo, p.n, p.hs.nconv, p.r0);
    else
        k_sum_columns<<<304, 256, 0, s>>>(p.V, p.ld, p.n, 1, p.r0);
    launch_counter() += 1;
}

// FP64 Rayleigh-Ritz of the FP32 phase's k converged pairs (vout[:, 0:k)):
// W = A Y with the FP64 operator, G = Y^T W, G = Z Theta Z^T (host Jacobi),
// Y' = Y Z, and the FP64 residuals of (theta_i, y'_i) (the reference's Ritz
// post-processing on its converged basis, HLanc.hpp:1765-1843, with true
// residuals for its Ritz estimates, H:1693-1695).  The refined pairs replace
// vout[:, 0:k) and the values in either case; *accepted when every residual
// is <= tol ||A||_inf.  *resid_max is the largest residual / ||A||_inf.
int refine_rr(Engine &E, ProbRes &p, double tol, bool *accepted, double *resid_max, long long *spmv_add) {
    *accepted = false;
    *resid_max = -1.0;
    *spmv_add = 0;
    const int k = p.hs.nconv, n = p.n, ldo = p.ldo;
    hlanc_csr_s *c = p.csr;
    if (!c || k < 1 || k > 64 || !p.vout) return HLANC_OK;
    cudaStream_t s = E.stream;
    const int nb = gram_blocks(n);
    struct Tmp {
        double *W = nullptr, *part = nullptr, *small = nullptr;
        ~Tmp() { if (W) cudaFree(W); if (part) cudaFree(part); if (small) cudaFree(small); }
    } t;
    CK(cudaMalloc(&t.W, sizeof(double) * (size_t)ldo * k));
    CK(cudaMalloc(&t.part, sizeof(double) * (size_t)nb * k * k));
    CK(cudaMalloc(&t.small, sizeof(double) * (2 * (size_t)k * k + 5 * (size_t)k)));
    double *G = t.small, *Zd = G + k * k, *th = Zd + k * k, *out4 = th + k;
    const int nst = (int)c->stiles_h.size();
    for (int i = 0; i < k; ++i)
        launch_spmv(c->rp_d, c->ci_d, c->val_d, c->sell(), c->stiles_d, nst, p.vout + (size_t)i * ldo,
                    t.W + (size_t)i * ldo, s);
    launch_gram(p.vout, t.W, n, ldo, k, t.part, G, s);
    std::vector<double> g((size_t)k * k), z((size_t)k * k), w(k), r4(4 * (size_t)k);
    CK(cudaMemcpyAsync(g.data(), G, sizeof(double) * k * k, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int j = 0; j < k; ++j)
        for (int i = 0; i < j; ++i) {
            const double a = 0.5 * (g[i + (size_t)j * k] + g[j + (size_t)i * k]);
            g[i + (size_t)j * k] = g[j + (size_t)i * k] = a;
        }
    if (host::sym_eig_jacobi(k, g.data(), w.data(), z.data())) return HLANC_OK;
    CK(cudaMemcpyAsync(Zd, z.data(), sizeof(double) * k * k, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(th, w.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    launch_rotate(p.vout, n, ldo, k, Zd, t.W, s);
    launch_residuals(c->rp_d, c->ci_d, c->val_d, n, k, th, t.W, ldo, out4, s);
    CK(cudaMemcpyAsync(r4.data(), out4, sizeof(double) * 4 * k, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpy2DAsync(p.vout, sizeof(double) * ldo, t.W, sizeof(double) * ldo, sizeof(double) * n, k,
                         cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(p.small + SM_VALS(p.ncv), th, sizeof(double) * k, cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
    CK(cudaGetLastError());
    *spmv_add = 2LL * k;
    double mx = 0.0;
    for (int i = 0; i < k; ++i) mx = std::max(mx, sqrt(r4[4 * (size_t)i]));
    const double na = c->norm_inf > 0 ? c->norm_inf : 1.0;
    *resid_max = mx / na;
    for (int i = 0; i < k; ++i) p.values[i] = w[i];
    *accepted = tol > 0.0 && mx <= tol * na;
    return HLANC_OK;
}

// Full solve of one problem.  values/vectors are host (device_out = false)
// or device pointers.
int solve_one(int dev, int n, int nev, int ncv, double *values, double *vectors, int ldv, bool device_out,
              hlanc_csr_s *csr, hlanc_host_op_fn host_op, void *host_ctx, const hlanc_opts_t &o,
              hlanc_stats_t *stats) {
    const double t0 = now_s();
    DevGuard g(dev);
    std::unique_ptr<Profiler> prof;
    if (o.profile) {
        prof.reset(new Profiler());
        g_prof = prof.get();
    }
    struct ProfReset { ~ProfReset() { g_prof = nullptr; } } prof_reset;
    Engine E;
    int rc = E.init(dev, o.stream, o.use_graphs != 0, o.restart_on_device != 0);
    if (rc) return rc;
    E.basis_tc = o.basis_kernel != HLANC_BASIS_FP64;
    E.cgs_mode = o.cgs_kernel;
    E.cycle_mode = o.cycle_kernel;
    const bool fp32 = csr && o.precision == HLANC_PREC_FP32_REFINE && csr->val32_d;
    int idx = 0;
    const hlanc_opts_t o1 = fp32 ? fp32_phase_opts(o) : o;
    rc = E.add(n, nev, ncv, csr, host_op, host_ctx, fp32 ? 1 : 0, o1, &idx);
    if (rc) return rc;
    E.active = {idx};
    if ((rc = E.upload())) return rc;
    if ((rc = E.start_vector(idx, o))) return rc;
    if ((rc = E.norm_init())) return rc;
    if ((rc = drive(E))) return rc;
    ProbRes &p = E.probs[idx];
    State S1 = p.hs;
    int refine_restarts = 0;
    State S = S1;
    bool accepted = false;             // the refined FP32-phase pairs are the result
    double rr_resid = -1.0;
    double copy_s = 0.0;               // host outputs: the copy-out of the pairs
    if (fp32) {
        // FP64 Rayleigh-Ritz of the FP32 phase's pairs; FP64 restart cycles
        // from the refined vectors where a residual misses the tolerance
        if (S1.status == ST_CONVERGED) {
            if ((rc = E.finalize(idx))) return rc;
            if (p.hs.status == ST_CONVERGED && p.hs.fin == 2) {
                long long rr_spmv = 0;
                if ((rc = refine_rr(E, p, o.tol, &accepted, &rr_resid, &rr_spmv))) return rc;
                S1.spmv += rr_spmv;
            }
        }
    }
    if (fp32 && accepted) {
        S = p.hs;
        S.spmv = S1.spmv;
    } else if (fp32) {
        fp64_phase_start(p, E.stream);
        State S0 = initial_state(nev, ncv, o);
        p.hs = S0;
        p.cycles = 0;
        CK(cudaMemcpyAsync(p.st, &S0, sizeof S0, cudaMemcpyHostToDevice, E.stream));
        p.fp32 = 0;
        if ((rc = E.upload())) return rc;
        if ((rc = E.norm_init())) return rc;
        if ((rc = drive(E))) return rc;
        S = p.hs;
        refine_restarts = S.iter;
        S.spmv += S1.spmv;
        S.passes += S1.passes;
        S.sumc += S1.sumc;
        S.sumt += S1.sumt;
        S.sumnev += S1.sumnev;
        S.napply += S1.napply;
    }
    int status = map_status(S.status);
    if (S.status == ST_CONVERGED && accepted) {
        // the refined pairs are in the library's vout and SM_VALS
        const int m = p.ncv, nconv = p.hs.nconv;
        if (device_out) {
            CK(cudaMemcpyAsync(values, p.small + SM_VALS(m), sizeof(double) * nconv, cudaMemcpyDeviceToDevice, E.stream));
            CK(cudaMemcpy2DAsync(vectors, sizeof(double) * (size_t)ldv, p.vout, sizeof(double) * (size_t)p.ldo,
                                 sizeof(double) * (size_t)n, m, cudaMemcpyDeviceToDevice, E.stream));
        } else {
            CK(cudaStreamSynchronize(E.stream));
            const double tc = now_s();
            CK(cudaMemcpyAsync(values, p.small + SM_VALS(m), sizeof(double) * nconv, cudaMemcpyDeviceToHost, E.stream));
            if ((rc = copy_d2h_2d(vectors, sizeof(double) * (size_t)ldv, p.vout, sizeof(double) * (size_t)p.ldo,
                                  sizeof(double) * (size_t)n, m, E.stream)))
                return rc;
            copy_s = now_s() - tc;
        }
        CK(cudaStreamSynchronize(E.stream));
    } else if (S.status == ST_CONVERGED) {
        if (device_out) {
            if (p.own_vout && p.vout) cudaFree(p.vout);
            p.vout = vectors;
            p.ldo = ldv;
            p.own_vout = false;
        }
        if ((rc = E.finalize(idx))) return rc;
        if (p.hs.status != ST_CONVERGED) {
            status = HLANC_NOT_CONVERGED;
        } else {
            const int m = p.ncv;
            const int nconv = p.hs.nconv;
            if (device_out) {
                CK(cudaMemcpyAsync(values, p.small + SM_VALS(m), sizeof(double) * nconv, cudaMemcpyDeviceToDevice, E.stream));
            } else {
                CK(cudaStreamSynchronize(E.stream));
                const double tc = now_s();
                CK(cudaMemcpyAsync(values, p.small + SM_VALS(m), sizeof(double) * nconv, cudaMemcpyDeviceToHost, E.stream));
                if ((rc = copy_d2h_2d(vectors, sizeof(double) * (size_t)ldv, p.vout, sizeof(double) * (size_t)p.ldo,
                                      sizeof(double) * (size_t)n, m, E.stream)))
                    return rc;
                copy_s = now_s() - tc;
            }
            CK(cudaStreamSynchronize(E.stream));
        }
    }
    const double nnz = csr ? (double)csr->nnz : 0.0;
    fill_stats(stats, S, p, nnz, fp32 ? 1 : 0, refine_restarts, now_s() - t0, status);
    if (stats) {
        stats->refine_residual = rr_resid;
        stats->copy_out_seconds = copy_s;
    }
    if (stats && S.status == ST_CONVERGED) stats->bytes_restart += 16.0 * n * ncv;
    fill_profile(S, p, nnz, fp32 ? 1 : 0);
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
    case HLANC_ERR_IO: return "file open/parse/write error";
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

long long hlanc_kernel_launches(void) { return launch_counter().load(); }

long long hlanc_kernel_launches_of(int kind) {
    if (kind == HLANC_KL_ALL) return launch_counter().load();
    if (kind < 0 || kind >= HLANC_KL_KINDS) return -1;
    return variant_counter(kind).load();
}

void hlanc_opts_default(hlanc_opts_t *o) {
    memset(o, 0, sizeof(*o));
    o->tol = 0.0;
    o->max_restarts = 200;
    o->precision = HLANC_PREC_FP64;
    o->seed = 0;
    o->start = nullptr;
    o->stream = nullptr;
    o->use_graphs = 1;
    o->restart_on_device = 0;
    o->profile = 0;
    o->basis_kernel = HLANC_BASIS_AUTO;
    o->cgs_kernel = HLANC_CGS_AUTO;
    o->wait_limit = 0;
    o->cycle_kernel = HLANC_CYCLE_AUTO;
}

int hlanc_last_profile(hlanc_profile_t *out) {
    if (!out || !g_have_prof) return HLANC_ERR_INVALID;
    *out = g_last_prof;
    return HLANC_OK;
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
    // The checks and the norm scan over row chunks on the host worker pool
    // (a 4.1M-row, 28.5M-entry matrix is ~30 ms of one core): row_ptr is
    // checked everywhere before any chunk reads col through it.
    const int nchunk = nrows >= (1 << 16) ? 64 : 1;
    auto chunk_rows = [&](int q, int &r0, int &r1) {
        r0 = (int)((long long)nrows * q / nchunk);
        r1 = (int)((long long)nrows * (q + 1) / nchunk);
    };
    std::vector<int> bad(nchunk, 0);
    HostPool::get().run(nchunk, [&](int q) {
        int r0, r1;
        chunk_rows(q, r0, r1);
        for (int r = r0; r < r1; ++r)
            if (row_ptr[r + 1] < row_ptr[r]) { bad[q] = 1; return; }
    });
    for (int q = 0; q < nchunk; ++q)
        if (bad[q]) return HLANC_ERR_INVALID;
    if (row_ptr[nrows] > nnz) return HLANC_ERR_INVALID;
    HostPool::get().run(nchunk, [&](int q) {
        int r0, r1;
        chunk_rows(q, r0, r1);
        for (int i = row_ptr[r0]; i < row_ptr[r1]; ++i)
            if (col[i] < 0 || col[i] >= ncols) { bad[q] = 1; return; }
    });
    for (int q = 0; q < nchunk; ++q)
        if (bad[q]) return HLANC_ERR_INVALID;
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
    std::vector<double> cn(nchunk, 0.0);
    std::vector<long long> cm(nchunk, 0);
    HostPool::get().run(nchunk, [&](int q) {
        int r0, r1;
        chunk_rows(q, r0, r1);
        double ninf = 0.0;
        long long mrow = 0;
        for (int r = r0; r < r1; ++r) {
            double s = 0.0;
            for (int i = grp[r]; i < grp[r + 1]; ++i) s += fabs(gva[i]);
            ninf = std::max(ninf, s);
            mrow = std::max<long long>(mrow, grp[r + 1] - grp[r]);
        }
        cn[q] = ninf;
        cm[q] = mrow;
    });
    h->norm_inf = *std::max_element(cn.begin(), cn.end());
    h->max_row = *std::max_element(cm.begin(), cm.end());
    build_spmv_tiles(grp, nrows, h->stiles_h);
    DevGuard g(dev);
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    const size_t nz = (size_t)std::max<long long>(gnnz, 1);
    CK(cudaMalloc(&h->rp_d, sizeof(int) * ((size_t)nrows + 1)));
    CK(cudaMalloc(&h->ci_d, sizeof(int) * nz + 16));
    CK(cudaMalloc(&h->val_d, sizeof(double) * nz + 16));
    CK(cudaMalloc(&h->xs_d, sizeof(double) * (size_t)std::max(ncols, 1)));
    CK(cudaMalloc(&h->ys_d, sizeof(double) * (size_t)std::max(nrows, 1)));
    CK(cudaMalloc(&h->stiles_d, sizeof(SpmvTile) * std::max<size_t>(h->stiles_h.size(), 1)));
    if (!h->stiles_h.empty())
        CK(cudaMemcpyAsync(h->stiles_d, h->stiles_h.data(), sizeof(SpmvTile) * h->stiles_h.size(),
                           cudaMemcpyHostToDevice, h->stream));
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
    int rc = autotune_spmv(h.get(), grp);
    if (rc) return rc;
    *out = h.release();
    return HLANC_OK;
}

int hlanc_csr_tuning(hlanc_csr_t h, int *rows_per_unit, int *lanes4_mean, int *lanes8_mean, double *us_default,
                     double *us_chosen) {
    if (!h) return HLANC_ERR_INVALID;
    if (rows_per_unit) *rows_per_unit = h->tune[0];
    if (lanes4_mean) *lanes4_mean = h->tune[2];
    if (lanes8_mean) *lanes8_mean = h->tune[3];
    if (us_default) *us_default = h->tune_us_default;
    if (us_chosen) *us_chosen = h->tune_us;
    return HLANC_OK;
}

int hlanc_csr_destroy(hlanc_csr_t h) {
    if (!h) return HLANC_OK;
    {
        DevGuard g(h->dev);
        cudaFree(h->rp_d); cudaFree(h->ci_d); cudaFree(h->val_d);
        if (h->val32_d) cudaFree(h->val32_d);
        cudaFree(h->xs_d); cudaFree(h->ys_d);
        if (h->stiles_d) cudaFree(h->stiles_d);
        h->free_sell();
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

}  // extern "C"

int hlanc::csr_view_of(hlanc_csr_t h, hlanc::CsrView *out) {
    if (!h || !out) return HLANC_ERR_INVALID;
    out->dev = h->dev; out->nrows = h->nrows; out->ncols = h->ncols; out->nnz = h->nnz;
    out->rp_d = h->rp_d; out->ci_d = h->ci_d; out->val_d = h->val_d; out->stream = h->stream;
    return HLANC_OK;
}

extern "C" {

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
    launch_spmv(h->rp_d, h->ci_d, h->val_d, h->sell(), h->stiles_d, (int)h->stiles_h.size(), xx, yy, h->stream);
    CK(cudaGetLastError());
    if (yy != y) CK(cudaMemcpyAsync(y, yy, sizeof(double) * h->nrows, cudaMemcpyDefault, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return HLANC_OK;
}

int hlanc_csr_spmv_async(hlanc_csr_t h, const double *x_d, double *y_d, void *stream) {
    if (!h || !x_d || !y_d) return HLANC_ERR_INVALID;
    DevGuard g(h->dev);
    launch_spmv(h->rp_d, h->ci_d, h->val_d, h->sell(), h->stiles_d, (int)h->stiles_h.size(), x_d, y_d,
                (cudaStream_t)stream);
    CK(cudaGetLastError());
    return HLANC_OK;
}

int hlanc_csr_spmv_f32_async(hlanc_csr_t h, const float *x_d, float *y_d, void *stream) {
    if (!h || !x_d || !y_d) return HLANC_ERR_INVALID;
    if (!h->val32_d) return HLANC_ERR_INVALID;
    DevGuard g(h->dev);
    launch_spmv_f32(h->rp_d, h->ci_d, h->val32_d, h->sell(), h->stiles_d, (int)h->stiles_h.size(), x_d, y_d,
                    (cudaStream_t)stream);
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

int hlanc_residuals_host(hlanc_csr_t csr, int k, const double *values_h, const double *vectors_h, int ldv_h,
                         double *resid_h, double *rdiff_h) {
    if (!csr || k <= 0 || !values_h || !vectors_h || ldv_h < csr->nrows) return HLANC_ERR_INVALID;
    DevGuard g(csr->dev);
    const int n = csr->nrows;
    double *vals = nullptr, *vecs = nullptr;
    CK(cudaMalloc(&vals, sizeof(double) * (size_t)k));
    cudaError_t e = cudaMalloc(&vecs, sizeof(double) * (size_t)n * k);
    if (e == cudaSuccess) e = cudaMemcpyAsync(vals, values_h, sizeof(double) * k, cudaMemcpyHostToDevice, csr->stream);
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(vecs, sizeof(double) * n, vectors_h, sizeof(double) * ldv_h, sizeof(double) * n, k,
                              cudaMemcpyHostToDevice, csr->stream);
    int rc = e == cudaSuccess ? hlanc_residuals_device(csr, k, vals, vecs, n, resid_h, rdiff_h) : HLANC_ERR_CUDA;
    cudaFree(vals);
    if (vecs) cudaFree(vecs);
    return rc;
}

int hlanc_eigs_write(const char *filename, int nev, int n, const double *values, const double *vectors,
                     int ldv) {
    return HLanc::write_eigs(filename, nev, n, values, vectors, ldv);
}

int hlanc_eigs_info(const char *filename, int *nev, int *n) {
    if (!nev || !n) return HLANC_ERR_INVALID;
    FILE *fp = filename ? fopen(filename, "r") : nullptr;
    if (!fp) return HLANC_ERR_IO;
    const bool ok = fscanf(fp, "%d", nev) == 1 && fscanf(fp, "%d", n) == 1 && *nev >= 0 && *n >= 0;
    fclose(fp);
    return ok ? HLANC_OK : HLANC_ERR_IO;
}

int hlanc_eigs_read(const char *filename, double *values, double *vectors, int ldv) {
    HLanc::eigs_t e;
    int rc = e.load(filename);
    if (rc) return rc;
    if ((e.nev > 0 && !values) || (e.nev > 0 && e.n > 0 && (!vectors || ldv < e.n))) return HLANC_ERR_INVALID;
    if (e.nev > 0) memcpy(values, e.value.data(), sizeof(double) * e.nev);
    for (int c = 0; c < e.nev; ++c)
        memcpy(vectors + (size_t)c * ldv, e.vector.data() + (size_t)c * e.n, sizeof(double) * e.n);
    return HLANC_OK;
}

// ---- diagnostics: the CGS kernels alone ----------------------------------------------
static int diag_no_op(void *, const double *, double *) { return 1; }

int hlanc_diag_cgs(int dev, int n, int c, int cgs_kernel, int reps, double *ms3) {
    if (n < 1024 || c < 2 || c > HLANC_MAX_NCV || reps < 1 || !ms3) return HLANC_ERR_INVALID;
    if (cgs_kernel != HLANC_CGS_FP64 && cgs_kernel != HLANC_CGS_HYBRID) return HLANC_ERR_INVALID;
    DevGuard g(dev);
    Engine E;
    int rc = E.init(dev, nullptr, false, false);
    if (rc) return rc;
    hlanc_opts_t o;
    hlanc_opts_default(&o);
    int idx = -1;
    rc = E.add(n, 1, c, nullptr, diag_no_op, nullptr, 0, o, &idx);
    if (rc) return rc;
    E.active.assign(1, idx);
    rc = E.upload();
    if (rc) return rc;
    ProbRes &p = E.probs[idx];
    // basis entries U(-1,1) sqrt(3/n) (columns of norm ~1), w entries U(-1,1)
    launch_diag_fill(p.V, (size_t)p.ld * c, sqrt(3.0 / n), 11, E.stream);
    launch_diag_fill(p.r0, (size_t)p.ld, 1.0, 12, E.stream);
    launch_diag_fill(p.r1, (size_t)p.ld, 1.0, 13, E.stream);
    // step 0 of an extension at j = c - 1 (c basis columns), second pass flagged
    State S = p.hs;
    S.status = ST_RUNNING;
    S.phase = PH_EXTEND;
    S.k = c - 1;
    S.np = 1;
    S.iter = 0;
    S.need2 = 1;
    S.need3 = 0;
    S.rnorm = S.wnorm = sqrt((double)n);
    CK(cudaMemcpyAsync(p.st, &S, sizeof S, cudaMemcpyHostToDevice, E.stream));
    struct Events {
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        ~Events() {
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
        }
    } ev;
    CK(cudaEventCreate(&ev.e0));
    CK(cudaEventCreate(&ev.e1));
    cudaEvent_t e0 = ev.e0, e1 = ev.e1;
    const bool hy = cgs_kernel == HLANC_CGS_HYBRID;
    const int pass_of[3] = {1, 2, 2}, which_of[3] = {0, 0, 1};
    // update coefficients at the level of a second pass (1e-13 ||w||), so the
    // FP32-copy update reads the copy for every column
    std::vector<double> hsmall((size_t)c);
    for (int i = 0; i < c; ++i) hsmall[i] = 1e-13 * sqrt((double)n) * (((i * 7) % 5) - 2) / 2.0;
    for (int q = 0; q < 3; ++q) {
        if (which_of[q] == 1)
            CK(cudaMemcpyAsync(p.small + SM_HV(c), hsmall.data(), sizeof(double) * c, cudaMemcpyHostToDevice,
                               E.stream));
        for (int w = 0; w < 2; ++w)
            launch_cgs_kernel(E.P_d, E.T_d, E.ntiles, E.one(), E.one_tr, 0, pass_of[q], which_of[q], hy, E.stream);
        CK(cudaEventRecord(e0, E.stream));
        for (int r = 0; r < reps; ++r)
            launch_cgs_kernel(E.P_d, E.T_d, E.ntiles, E.one(), E.one_tr, 0, pass_of[q], which_of[q], hy, E.stream);
        CK(cudaEventRecord(e1, E.stream));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        ms3[q] = ms / reps;
    }
    CK(cudaGetLastError());
    return HLANC_OK;
}

// ---- batched solves ------------------------------------------------------------------
}  // extern "C"

struct hlanc_batch_s {
    Engine E;
    std::vector<int> idx;
    std::vector<hlanc_csr_s *> ops;
    std::vector<int> nev, ncv;
    hlanc_opts_t o;
    int dev = 0;
};

namespace {

// Drive a set of problems; with FP32 operators, a second FP64 phase starts
// each from its FP32 phase (fp64_phase_start).
int run_problems(Engine &E, const std::vector<int> &idx, const std::vector<int> &nev, const std::vector<int> &ncv,
                 const hlanc_opts_t &o, bool fp32, std::vector<State> &first_phase) {
    int rc;
    E.active = idx;
    if ((rc = E.upload())) return rc;
    for (int p : idx)
        if ((rc = E.start_vector(p, o))) return rc;
    if ((rc = E.norm_init())) return rc;
    if ((rc = drive(E))) return rc;
    first_phase.clear();
    for (int p : idx) first_phase.push_back(E.probs[p].hs);
    if (!fp32) return HLANC_OK;
    std::vector<int> conv;
    for (int p : idx)
        if (E.probs[p].hs.status == ST_CONVERGED) conv.push_back(p);
    if (!conv.empty() && (rc = E.finalize_many(conv))) return rc;
    for (size_t q = 0; q < idx.size(); ++q) {
        ProbRes &p = E.probs[idx[q]];
        fp64_phase_start(p, E.stream);
        State S0 = initial_state(nev[q], ncv[q], o);
        p.hs = S0;
        p.cycles = 0;
        p.fp32 = 0;
        CK(cudaMemcpyAsync(p.st, &S0, sizeof S0, cudaMemcpyHostToDevice, E.stream));
    }
    if ((rc = E.upload())) return rc;
    if ((rc = E.norm_init())) return rc;
    return drive(E);
}

}  // namespace

extern "C" {

int hlanc_batch_create(int dev, int nprob, const hlanc_csr_t *ops, const int *nev, const int *ncv,
                       const hlanc_opts_t *opts, hlanc_batch_t *out) {
    if (nprob <= 0 || !ops || !nev || !ncv || !out) return HLANC_ERR_INVALID;
    std::unique_ptr<hlanc_batch_s> b(new hlanc_batch_s());
    if (opts) b->o = *opts;
    else hlanc_opts_default(&b->o);
    b->dev = dev;
    DevGuard g(dev);
    int rc = b->E.init(dev, b->o.stream, b->o.use_graphs != 0, b->o.restart_on_device != 0);
    if (rc) return rc;
    b->E.basis_tc = b->o.basis_kernel != HLANC_BASIS_FP64;
    b->E.cgs_mode = b->o.cgs_kernel;
    b->E.cycle_mode = b->o.cycle_kernel;
    if (nprob > 1) b->E.min_tile_rows = BATCH_MIN_TILE_ROWS;
    const bool fp32 = b->o.precision == HLANC_PREC_FP32_REFINE;
    const hlanc_opts_t o1 = fp32 ? fp32_phase_opts(b->o) : b->o;
    for (int i = 0; i < nprob; ++i) {
        hlanc_csr_s *c = ops[i];
        if (!c || c->dev != dev) return HLANC_ERR_INVALID;
        if ((rc = validate(c->nrows, nev[i], ncv[i], c->nrows))) return rc;
        if (c->ncols > c->nrows) return HLANC_ERR_INVALID;
        if (fp32 && !c->val32_d) return HLANC_ERR_INVALID;
        int idx = 0;
        if ((rc = b->E.add(c->nrows, nev[i], ncv[i], c, nullptr, nullptr, fp32 ? 1 : 0, o1, &idx))) return rc;
        b->idx.push_back(idx);
        b->ops.push_back(c);
        b->nev.push_back(nev[i]);
        b->ncv.push_back(ncv[i]);
    }
    *out = b.release();
    return HLANC_OK;
}

int hlanc_batch_run(hlanc_batch_t b, double **values_d, double **vectors_d, int *status, hlanc_stats_t *stats) {
    if (!b || !values_d || !vectors_d) return HLANC_ERR_INVALID;
    const double t0 = now_s();
    DevGuard g(b->dev);
    std::unique_ptr<Profiler> prof;
    if (b->o.profile) {
        prof.reset(new Profiler());
        g_prof = prof.get();
    }
    struct ProfReset { ~ProfReset() { g_prof = nullptr; } } prof_reset;
    Engine &E = b->E;
    const bool fp32 = b->o.precision == HLANC_PREC_FP32_REFINE;
    std::vector<State> first;
    int rc = run_problems(E, b->idx, b->nev, b->ncv, b->o, fp32, first);
    if (rc) return rc;
    std::vector<int> conv;
    for (size_t q = 0; q < b->idx.size(); ++q) {
        ProbRes &p = E.probs[b->idx[q]];
        if (p.own_vout && p.vout) cudaFree(p.vout);
        p.vout = vectors_d[q];
        p.ldo = p.n;
        p.own_vout = false;
        if (p.hs.status == ST_CONVERGED) conv.push_back(b->idx[q]);
    }
    if (!conv.empty() && (rc = E.finalize_many(conv))) return rc;
    long long spmv = 0, passes = 0;
    int ok = 0, restarts = 0;
    double by_spmv = 0, by_cgs = 0, by_rs = 0;
    for (size_t q = 0; q < b->idx.size(); ++q) {
        ProbRes &p = E.probs[b->idx[q]];
        State S = p.hs;
        if (fp32) {
            S.spmv += first[q].spmv; S.passes += first[q].passes; S.sumc += first[q].sumc; S.sumt += first[q].sumt;
            S.sumnev += first[q].sumnev; S.napply += first[q].napply;
        }
        const int st = map_status(S.status);
        if (status) status[q] = st;
        if (S.status == ST_CONVERGED) {
            ++ok;
            CK(cudaMemcpyAsync(values_d[q], p.small + SM_VALS(p.ncv), sizeof(double) * S.nconv,
                               cudaMemcpyDeviceToDevice, E.stream));
        }
        hlanc_stats_t one;
        fill_stats(&one, S, p, (double)b->ops[q]->nnz, fp32 ? 1 : 0, 0, 0.0, st);
        spmv += one.spmv_calls; passes += one.cgs_passes; restarts = std::max(restarts, one.restarts);
        by_spmv += one.bytes_spmv; by_cgs += one.bytes_cgs; by_rs += one.bytes_restart;
    }
    CK(cudaStreamSynchronize(E.stream));
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->spmv_calls = spmv; stats->cgs_passes = passes; stats->restarts = restarts;
        stats->nconv = ok; stats->status = ok == (int)b->idx.size() ? HLANC_OK : HLANC_NOT_CONVERGED;
        stats->seconds = now_s() - t0;
        stats->bytes_spmv = by_spmv; stats->bytes_cgs = by_cgs; stats->bytes_restart = by_rs;
    }
    return ok == (int)b->idx.size() ? HLANC_OK : HLANC_NOT_CONVERGED;
}

int hlanc_batch_destroy(hlanc_batch_t b) {
    if (!b) return HLANC_OK;
    int dev = b->dev;
    {
        DevGuard g(dev);
        delete b;
    }
    return HLANC_OK;
}

}  // extern "C"

// ---- serving: continuous batching --------------------------------------------------
// Resident solves are spread over lanes.  A lane is an Engine with its own
// stream, launch tables and mailbox, so a step can finish one lane's cycle on
// the host (restart decisions, finalisation, retirement, admission) while the
// other lanes' cycles run on the device, then launch that lane's next cycle
// without waiting for it.  Ritz vectors of a converged solve are computed in
// its lane's next cycle; problem memory comes from a stream-ordered pool, so
// admitting and retiring solves never synchronises the device.
struct hlanc_server_s {
    struct Request {
        long long id = 0;
        hlanc_csr_s *csr = nullptr;
        int nev = 0, ncv = 0;
        hlanc_opts_t o;
        int state = 0;             // 0 pending, 1 resident, 2 done
        int status = HLANC_OK;
        int lane = -1, prob = -1;
        size_t bytes = 0;
        double work = 0.0;         // n * ncv, balances the lanes
        bool cancel = false;
        bool fresh = false;        // start vector pending
        bool need_norm = false;    // start-vector norm pending
        bool push_state = false;   // host State must reach the device (phase switch)
        bool finishing = false;    // finalised on the host; Ritz vectors in the next cycle
        std::vector<double> values, vectors, Q2, start;
        hlanc_stats_t stats;
        double t_submit = 0, t_admit = 0, t_done = 0;
        int phase = 0;             // 1: FP32-SpMV phase of a mixed-precision solve, 0: FP64
        State first;               // counters of the FP32 phase
    };
    struct Lane {
        Engine E;
        std::vector<long long> ids;      // resident requests, in slot order
        bool inflight = false, dirty = true;
        double work = 0.0;
        cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    };
    hlanc_server_opts_t opts;
    cudaMemPool_t pool = nullptr;
    std::vector<std::unique_ptr<Lane>> lanes;
    std::map<long long, Request> reqs;
    std::deque<long long> pending;
    int resident = 0;
    size_t used = 0;
    long long next_id = 1;
    hlanc_server_stats_t st;
    std::mutex mu;

    ~hlanc_server_s() {
        for (auto &L : lanes) {
            if (L->E.stream) cudaStreamSynchronize(L->E.stream);
            if (L->ev0) cudaEventDestroy(L->ev0);
            if (L->ev1) cudaEventDestroy(L->ev1);
        }
        lanes.clear();                    // frees go to the pool on the lane streams
        if (pool) cudaMemPoolDestroy(pool);   // released once those frees complete
    }
};

namespace {

using Srv = hlanc_server_s;

// Record a request's result and retire its problem (not its slot in L.ids).
void srv_finish(Srv &s, Srv::Lane &L, Srv::Request &r, int status) {
    ProbRes &p = L.E.probs[r.prob];
    State S = p.hs;
    int refine = 0;
    const bool mixed = r.o.precision == HLANC_PREC_FP32_REFINE;
    if (mixed) {
        refine = S.iter;
        S.spmv += r.first.spmv; S.passes += r.first.passes; S.sumc += r.first.sumc; S.sumt += r.first.sumt;
        S.sumnev += r.first.sumnev; S.napply += r.first.napply;
    }
    r.status = status;
    fill_stats(&r.stats, S, p, (double)r.csr->nnz, mixed, refine, 0.0, status);
    r.t_done = now_s();
    r.stats.seconds = r.t_done - r.t_submit;
    r.state = 2;
    L.E.retire(r.prob);
    s.used -= r.bytes;
    s.resident -= 1;
    L.work -= r.work;
    L.dirty = true;
    s.st.retired += 1;
}

// FP32 phase over: the FP64 phase starts from it (fp64_phase_start).
void srv_switch_to_fp64(Srv::Lane &L, Srv::Request &r) {
    ProbRes &p = L.E.probs[r.prob];
    r.first = p.hs;
    fp64_phase_start(p, L.E.stream);
    p.hs = initial_state(r.nev, r.ncv, r.o);
    p.cycles = 0;
    p.fp32 = 0;
    r.phase = 0;
    r.push_state = true;
    r.need_norm = true;
    L.dirty = true;                       // the descriptor drops its FP32 values
}

// Wait for the lane's cycle, then make every decision it enables.
int srv_complete(Srv &s, Srv::Lane &L) {
    if (!L.inflight) return HLANC_OK;
    Engine &E = L.E;
    double t = now_s();
    CK(cudaEventSynchronize(L.ev1));
    CK(cudaGetLastError());
    s.st.wait_ms += (now_s() - t) * 1e3;
    L.inflight = false;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, L.ev0, L.ev1) == cudaSuccess) s.st.gpu_ms += ms;
    E.unpack_mailbox();
    for (int pi : E.active) E.probs[pi].cycles += 1;
    s.st.cycles += 1;
    t = now_s();
    // Ritz vectors that the cycle produced
    std::vector<long long> keep;
    for (long long id : L.ids) {
        Srv::Request &r = s.reqs[id];
        ProbRes &p = E.probs[r.prob];
        if (p.hs.err != DEV_ERR_NONE) {            // a bounded device wait gave up
            r.finishing = false;
            p.hs.status = ST_FAILED;               // no host restart for it below
            p.hs.phase = PH_DONE;
            srv_finish(s, L, r, HLANC_ERR_DEVICE_TIMEOUT);
            continue;
        }
        if (!r.finishing) { keep.push_back(id); continue; }
        r.finishing = false;
        if (p.hs.fin != 2) {                       // not produced: report, do not guess
            srv_finish(s, L, r, HLANC_ERR_CUDA);
            continue;
        }
        if (r.phase == 1) {
            srv_switch_to_fp64(L, r);
            keep.push_back(id);
            continue;
        }
        const int n = p.n, m = p.ncv;
        r.values.assign(p.values.begin(), p.values.begin() + p.hs.nconv);
        r.vectors.resize((size_t)n * m);
        int rc;
        if ((rc = copy_d2h_2d(r.vectors.data(), sizeof(double) * n, p.vout, sizeof(double) * p.ldo,
                              sizeof(double) * n, m, E.stream)))
            return rc;
        srv_finish(s, L, r, HLANC_OK);
    }
    L.ids.swap(keep);
    // restart decisions of the problems that extended (slots of the last launch)
    int running, nev_max, np_max;
    E.host_restarts(&running, &nev_max, &np_max);
    // terminal states
    keep.clear();
    for (long long id : L.ids) {
        Srv::Request &r = s.reqs[id];
        ProbRes &p = E.probs[r.prob];
        if (r.cancel) {
            srv_finish(s, L, r, HLANC_ERR_CANCELLED);
            continue;
        }
        if (p.hs.status == ST_RUNNING || r.finishing || r.push_state) { keep.push_back(id); continue; }
        if (p.hs.status == ST_CONVERGED && p.hs.fin == 0) {
            host::FinalizeIO io;
            io.ncv = p.ncv; io.nev0 = p.hs.nev0; io.np0 = p.hs.np0; io.nconv = p.hs.nconv;
            io.tol = p.hs.tol; io.eps23 = p.hs.eps23;
            io.h = p.h.data(); io.ritz_s = p.ritz_s.data(); io.bnds_s = p.bnds_s.data();
            io.values = p.values.data();
            r.Q2.assign((size_t)p.ncv * p.ncv, 0.0);
            io.Q2 = r.Q2.data();
            if (host::finalize(io) == 0) {
                p.hs.fin = 1;
                r.finishing = true;
                keep.push_back(id);
                continue;
            }
            p.hs.status = ST_FAILED;
        }
        if (r.phase == 1) {                        // FP32 phase did not converge
            srv_switch_to_fp64(L, r);
            keep.push_back(id);
            continue;
        }
        srv_finish(s, L, r, map_status(p.hs.status));
    }
    L.ids.swap(keep);
    s.st.host_ms += (now_s() - t) * 1e3;
    return HLANC_OK;
}

// Admit pending requests into lane li while slots and memory allow and no
// other lane carries less work.
int srv_admit(Srv &s, int li) {
    Srv::Lane &L = *s.lanes[li];
    while (!s.pending.empty() && s.resident < s.opts.max_slots) {
        Srv::Request &r = s.reqs[s.pending.front()];
        if (r.cancel) {
            r.state = 2; r.status = HLANC_ERR_CANCELLED; r.t_done = now_s();
            s.pending.pop_front();
            continue;
        }
        if (s.used + r.bytes > s.opts.mem_budget_bytes) break;
        bool lighter_elsewhere = false;
        for (size_t o = 0; o < s.lanes.size(); ++o)
            if ((int)o != li && s.lanes[o]->work < L.work) lighter_elsewhere = true;
        if (lighter_elsewhere) break;
        const hlanc_opts_t o1 = r.phase == 1 ? fp32_phase_opts(r.o) : r.o;
        int idx = 0, rc;
        if ((rc = L.E.add(r.csr->nrows, r.nev, r.ncv, r.csr, nullptr, nullptr, r.phase, o1, &idx))) return rc;
        if ((rc = L.E.probs[idx].alloc_vout(L.E.stream))) return rc;
        r.prob = idx;
        r.lane = li;
        r.state = 1;
        r.t_admit = now_s();
        r.fresh = true;
        r.need_norm = true;
        s.used += r.bytes;
        s.resident += 1;
        L.work += r.work;
        L.ids.push_back(r.id);
        L.dirty = true;
        s.pending.pop_front();
        s.st.admitted += 1;
    }
    return HLANC_OK;
}

// Enqueue the lane's next cycle; returns without waiting for it.
int srv_launch(Srv &s, Srv::Lane &L) {
    Engine &E = L.E;
    if (L.ids.empty()) return HLANC_OK;
    double t = now_s();
    int rc;
    if (L.dirty) {
        E.active.clear();
        for (long long id : L.ids) E.active.push_back(s.reqs[id].prob);
        if ((rc = E.upload())) return rc;
        L.dirty = false;
    }
    s.st.admin_ms += (now_s() - t) * 1e3;
    t = now_s();
    // mailbox of this cycle, from the host mirrors
    int steps = 0, basis_nev = 0;
    bool ritz = false, norm = false;
    for (size_t a = 0; a < L.ids.size(); ++a) {
        Srv::Request &r = s.reqs[L.ids[a]];
        ProbRes &p = E.probs[r.prob];
        const int m = p.ncv;
        double *slot = E.mbox_h + E.off_h[a];
        E.flag_h[a] = 0;
        if (r.finishing) {
            memcpy(slot, &p.hs, sizeof(State));
            memcpy(slot + MBOX_STATE + 2 * m, r.Q2.data(), sizeof(double) * m * m);
            memcpy(slot + MBOX_STATE + 2 * m + (size_t)m * m, p.values.data(), sizeof(double) * m);
            E.flag_h[a] = 3;
            ritz = true;
        } else if (r.push_state) {
            memcpy(slot, &p.hs, sizeof(State));
            E.flag_h[a] = 2;
            r.push_state = false;
        } else if (p.cycles > 0 && p.hs.status == ST_RUNNING && p.hs.phase == PH_APPLY) {
            memcpy(slot, &p.hs, sizeof(State));
            memcpy(slot + MBOX_STATE, p.h.data(), sizeof(double) * 2 * m);
            memcpy(slot + MBOX_STATE + 2 * m, p.Q.data(), sizeof(double) * m * m);
            E.flag_h[a] = 1;
        }
        if (p.hs.status == ST_RUNNING) {
            steps = std::max(steps, p.cycles == 0 ? p.ncv : p.ncv - p.nev0);
            if (p.cycles > 0 && p.hs.phase == PH_APPLY) basis_nev = std::max(basis_nev, p.hs.nev);
        }
    }
    if ((rc = E.push_mailbox())) return rc;
    CK(cudaEventRecord(L.ev0, E.stream));
    const int na = (int)E.active.size();
    launch_scatter(E.P_d, na, E.off_d, E.flag_d, E.mbox_d, E.stream);
    for (long long id : L.ids) {
        Srv::Request &r = s.reqs[id];
        if (r.fresh) {
            hlanc_opts_t o = r.o;
            if (!r.start.empty()) o.start = r.start.data();
            if ((rc = E.start_vector(r.prob, o))) return rc;
            r.fresh = false;
        }
        norm = norm || r.need_norm;
        r.need_norm = false;
    }
    if (norm) launch_norm_init(E.P_d, E.T_d, E.ntiles, E.stream);
    if (ritz) launch_ritz(E.P_d, E.T_d, E.ntiles, E.max_ncv, E.basis_tc, E.stream);
    if (basis_nev > 0)
        launch_basis(E.P_d, E.T_d, E.ntiles, E.max_ncv, Engine::basis_bucket(basis_nev), E.basis_tc, E.stream);
    E.enqueue_steps(steps);
    launch_gather(E.P_d, na, E.off_d, E.mbox_d, E.stream);
    if ((rc = E.pull_async())) return rc;
    CK(cudaEventRecord(L.ev1, E.stream));
    CK(cudaGetLastError());
    L.inflight = true;
    s.st.launch_ms += (now_s() - t) * 1e3;
    return HLANC_OK;
}

}  // namespace

extern "C" {

int hlanc_server_create(const hlanc_server_opts_t *opts, hlanc_server_t *out) {
    if (!opts || !out || opts->max_slots <= 0 || opts->lanes < 0 || opts->lanes > 8) return HLANC_ERR_INVALID;
    std::unique_ptr<hlanc_server_s> s(new hlanc_server_s());
    s->opts = *opts;
    if (s->opts.lanes == 0) s->opts.lanes = 2;
    memset(&s->st, 0, sizeof s->st);
    DevGuard g(opts->dev);
    cudaMemPoolProps props;
    memset(&props, 0, sizeof props);
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = opts->dev;
    CK(cudaMemPoolCreate(&s->pool, &props));
    unsigned long long keep_all = ~0ULL;      // keep freed blocks for the next admissions
    CK(cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep_all));
    for (int i = 0; i < s->opts.lanes; ++i) {
        std::unique_ptr<hlanc_server_s::Lane> L(new hlanc_server_s::Lane());
        int rc = L->E.init(opts->dev, nullptr, false, false);   // the active set changes often: eager launches
        if (rc) return rc;
        L->E.pool = s->pool;
        L->E.min_tile_rows = SERVE_MIN_TILE_ROWS;
        CK(cudaEventCreate(&L->ev0));
        CK(cudaEventCreate(&L->ev1));
        s->lanes.push_back(std::move(L));
    }
    *out = s.release();
    return HLANC_OK;
}

int hlanc_server_submit(hlanc_server_t s, hlanc_csr_t csr, int nev, int ncv, const hlanc_opts_t *opts,
                        long long *request_id) {
    if (!s || !csr || !request_id) return HLANC_ERR_INVALID;
    int rc = validate(csr->nrows, nev, ncv, csr->nrows);
    if (rc) return rc;
    if (csr->dev != s->opts.dev || csr->ncols > csr->nrows) return HLANC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    hlanc_server_s::Request r;
    r.id = s->next_id++;
    r.csr = csr;
    r.nev = nev;
    r.ncv = ncv;
    if (opts) r.o = *opts;
    else hlanc_opts_default(&r.o);
    if (r.o.start) r.start.assign(r.o.start, r.o.start + csr->nrows);
    r.o.start = nullptr;
    const bool fp32 = r.o.precision == HLANC_PREC_FP32_REFINE && csr->val32_d;
    r.o.precision = fp32 ? HLANC_PREC_FP32_REFINE : HLANC_PREC_FP64;
    r.phase = fp32 ? 1 : 0;
    r.bytes = ProbRes::estimate(csr->nrows, ncv, fp32 ? 1 : 0, SERVE_MIN_TILE_ROWS);
    r.work = (double)csr->nrows * ncv;
    if (r.bytes > s->opts.mem_budget_bytes) return HLANC_ERR_ALLOC;
    r.t_submit = now_s();
    memset(&r.stats, 0, sizeof r.stats);
    *request_id = r.id;
    s->pending.push_back(r.id);
    s->reqs.emplace(r.id, std::move(r));
    return HLANC_OK;
}

// One scheduler step: every lane completes its cycle in flight, admits what
// fits and launches its next cycle.  While the host works on one lane, the
// other lanes' cycles run on the device.
int hlanc_server_step(hlanc_server_t s, int *n_active, int *n_pending) {
    if (!s) return HLANC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    DevGuard g(s->opts.dev);
    const double t0 = now_s();
    int rc;
    for (size_t li = 0; li < s->lanes.size(); ++li) {
        hlanc_server_s::Lane &L = *s->lanes[li];
        if ((rc = srv_complete(*s, L))) return rc;
        double t = now_s();
        if ((rc = srv_admit(*s, (int)li))) return rc;
        s->st.admin_ms += (now_s() - t) * 1e3;
        if ((rc = srv_launch(*s, L))) return rc;
    }
    s->st.steps += 1;
    s->st.wall_ms += (now_s() - t0) * 1e3;
    if (n_active) *n_active = s->resident;
    if (n_pending) *n_pending = (int)s->pending.size();
    return HLANC_OK;
}

int hlanc_server_poll(hlanc_server_t s, long long request_id, int *done, int *status, double *values,
                      double *vectors, hlanc_stats_t *stats) {
    if (!s || !done) return HLANC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(request_id);
    if (it == s->reqs.end()) return HLANC_ERR_INVALID;
    auto &r = it->second;
    *done = r.state == 2;
    if (!*done) return HLANC_OK;
    if (status) *status = r.status;
    if (values && !r.values.empty()) memcpy(values, r.values.data(), sizeof(double) * r.values.size());
    if (vectors && !r.vectors.empty()) memcpy(vectors, r.vectors.data(), sizeof(double) * r.vectors.size());
    if (stats) *stats = r.stats;
    return HLANC_OK;
}

int hlanc_server_cancel(hlanc_server_t s, long long request_id) {
    if (!s) return HLANC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(request_id);
    if (it == s->reqs.end()) return HLANC_ERR_INVALID;
    if (it->second.state != 2) it->second.cancel = true;
    return HLANC_OK;
}

int hlanc_server_stats(hlanc_server_t s, hlanc_server_stats_t *out) {
    if (!s || !out) return HLANC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    return HLANC_OK;
}

int hlanc_server_destroy(hlanc_server_t s) {
    if (!s) return HLANC_OK;
    const int dev = s->opts.dev;
    {
        DevGuard g(dev);
        delete s;
    }
    return HLANC_OK;
}

}  // extern "C"
