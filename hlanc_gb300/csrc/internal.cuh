// internal.cuh -- device data model of the GB300 IRLM engine.
//
// One solve (or one member of a batch) is a "problem".  Everything the
// implicitly restarted Lanczos loop touches lives in HBM for the whole solve:
//   V      ld x ncv FP64 basis, column-major, ld = n rounded up to 64 rows
//          (512-byte aligned columns; padding rows stay zero),
//   V32    its FP32 shadow, written wherever a column of V is written; the
//          CGS update reads it for the columns whose coefficient is so small
//          that FP32 products keep the update FP64-accurate (k_apply),
//   r0/r1  residual ping-pong (step j reads r[j&1], writes r[(j+1)&1]),
//   small  the ncv-sized arrays of the reference's workl (T, Ritz values,
//          bounds, Q), see the SM_* offsets,
//   State  scalars (rnorm, wnorm, DGKS flags, nev/np, status).
// Rows are split into tiles (multiples of 64 rows); every row-parallel kernel
// runs one CTA per tile and reduces its partial sums deterministically: each
// tile writes a fixed slot, the last CTA to finish sums the slots in tile
// order.  A batch is simply several problems whose tiles share one launch.
#pragma once

#include <atomic>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/hlanc_gb300.h"
#include "fixed_point.cuh"

namespace hlanc {

constexpr int TPB = 256;                 // threads per CTA of the tile kernels
constexpr int ROW_ALIGN = 64;            // tile boundaries / ld granularity
constexpr int MAXNCV = HLANC_MAX_NCV;
constexpr int LONG_ROW = 96;             // rows longer than this are reduced by a warp

enum : int { ST_RUNNING = 0, ST_CONVERGED = 1, ST_NOT_CONVERGED = 2, ST_FAILED = 3 };
enum : int { PH_EXTEND = 0, PH_APPLY = 1, PH_DONE = 2 };

struct State {
    int status;            // ST_*
    int phase;             // PH_*
    int k, np, nev;        // current extension runs steps j = k .. k+np-1; nev after adjustment
    int iter;              // restart cycles completed (ds_solver loop counter)
    int nconv;
    int need2, need3;      // DGKS second / third pass needed for the current step
    int max_iter;
    int nev0, np0, ncv;
    int err;               // DEV_ERR_*: a bounded device wait gave up (the solve is abandoned)
    double rnorm, wnorm;
    double tol, eps23;
    long long spmv, passes;
    long long sumc;        // sum over CGS passes of the column count c (algorithmic bytes)
    long long sumnev;      // sum over applied restarts of nev (algorithmic bytes)
    long long sumt;        // sum over CGS updates of the columns read from the FP32 shadow
    int napply;            // restarts applied to V
    int fin;               // 0 = not finalised, 1 = Qfull/values ready, 2 = Ritz vectors written
    int wait_limit;        // polls of a bounded device wait (0: WAIT_LIMIT_DEFAULT, < 0: none)
};

// Error codes a kernel leaves in State::err (the host returns them as
// HLANC_ERR_DEVICE_TIMEOUT).
enum : int { DEV_ERR_NONE = 0, DEV_ERR_MMA_WAIT = 1, DEV_ERR_GRID_WAIT = 2 };
constexpr int WAIT_LIMIT_DEFAULT = 1 << 20;   // far above any real wait

// offsets (in doubles) of the per-problem small arrays, m = ncv
__host__ __device__ inline int SM_H(int)        { return 0; }           // h[j]=beta_j, h[m+j]=alpha_j
__host__ __device__ inline int SM_HV(int m)     { return 2 * m; }       // projection coefficients
__host__ __device__ inline int SM_RITZ(int m)   { return 3 * m; }
__host__ __device__ inline int SM_BOUNDS(int m) { return 4 * m; }
__host__ __device__ inline int SM_RITZS(int m)  { return 5 * m; }       // last-iteration snapshot (workl+ncv)
__host__ __device__ inline int SM_BNDS(int m)   { return 6 * m; }       // (workl+2ncv)
__host__ __device__ inline int SM_VALS(int m)   { return 7 * m; }       // final eigenvalues
__host__ __device__ inline int SM_WORK(int m)   { return 8 * m; }       // 4m scratch
__host__ __device__ inline int SM_Q(int m)      { return 12 * m; }      // m*m (dsapps Q / eigvecs of T)
__host__ __device__ inline int SM_Q2(int m)     { return 12 * m + m * m; }  // m*m (final Householder Q)
__host__ __device__ inline int SM_SIZE(int m)   { return 12 * m + 2 * m * m; }

// Sliced-ELL copy of a matrix's rows of at most LONG_ROW entries (kind 5
// units; row0/row1 are slice indices, SELL_SLICES_PER_UNIT slices per
// unit).  Rows are sorted by length inside windows of SELL_SIGMA rows and
// packed SELL_C to a slice; element k of lane l of slice s sits at
// ptr[s] + k * SELL_C + l (padding: column 0, value 0), so a warp walks
// 32 rows of nearly equal length with coalesced loads and every FP64 FMA
// slot does useful work.  row[s * SELL_C + l] is the lane's row (-1: none).
constexpr int SELL_C = 32;
constexpr int SELL_SIGMA = 1024;
constexpr int SELL_SLICES_PER_UNIT = 8;   // = TPB / 32: one warp per slice
struct Sell {
    const long long *ptr;
    const int *len;
    const int *row;
    const int *col;
    const double *val;
    const float *val32;
};

struct Problem {
    // operator (general CSR on the device)
    const int *row_ptr;
    const int *col;
    const double *val;
    const float *val32;    // FP32 values (mixed precision), or null
    int n, ld, ncv, nev0;
    int tile0, ntiles;
    int fp32;              // SpMV on FP32 values/vectors
    int pstride;           // values per tile partial slot (part is pstride x ntiles, value-major)
    double *V;
    float *V32;            // FP32 shadow of V (same layout), read by the CGS update (k_apply)
    double *r0, *r1;
    double *part;          // tile partial sums, value-major (pstride x ntiles)
    double *gpart;         // group partial sums, value-major (pstride x ngroups)
    unsigned *counter;     // [0] problem counter, [1 + g] group counters
    State *st;
    double *small;
    const double *wext;    // non-null: operator output is supplied by the host callback path
    double *vout;          // Ritz vectors destination (device, ldo x ncv)
    int ldo, pad2;
    Sell sell;             // sliced-ELL rows of the operator (kind 5 SpMV units), or null pointers
};

struct Tile { int prob, row0, row1, pad; };

// SpMV work units, built once per operator from the row lengths:
//   kind 0 (short):  up to SPMV_ROWS consecutive rows of <= LONG_ROW entries
//                    and <= SPMV_NNZ entries in total; thread per row;
//   kind 1 (medium): up to TPB/16 consecutive rows of LONG_ROW..WIDE_ROW
//                    entries; 16 lanes per row (measured on GB300: 5.6% faster
//                    in the solver than a warp per row on the power-law graph);
//   kind 2 (wide):   one row of more than WIDE_ROW entries; whole CTA;
//   kind 3 / 4:      a short-row unit whose mean row length is above
//                    SUBWARP4_MEAN / SUBWARP8_MEAN: 4 / 8 lanes per row.
// Balancing by entries keeps skewed (power-law) matrices from piling their
// long rows onto a few CTAs, and no CTA waits on a barrier for one warp.
// 1024-row units amortise each CTA's start-up loads (measured 24% faster
// than 256-row units on the 4.1M-row Laplacian, equal on the power-law graph).
constexpr int SPMV_ROWS = 1024;
constexpr int SPMV_NNZ = 16384;
constexpr int WIDE_ROW = 2048;
// Measured on GB300 (power-law graph, n = 2^22, median row 18 entries):
// 4 / 8 lanes per row above a mean of 12 / 32 entries took the standalone
// SpMV from 828 to 644 us (in the solver 877 -> 776 us); 8/24, 12/20 and
// 16/- were slower, and the 7-entry Laplacian rows keep thread per row.
constexpr int SUBWARP4_MEAN = 12;
constexpr int SUBWARP8_MEAN = 32;
struct SpmvTile { int prob, row0, row1, kind; };


// ---- device helpers --------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Reduce 8 values per lane across the warp ("transposed" butterfly): 9
// FP64 adds per lane instead of 8 x 5.  On return lane l holds the warp sum
// of value q = l >> 2 (lanes 4q..4q+3 hold the same value).  Fixed order,
// so results are deterministic.
__device__ __forceinline__ double warp_reduce8(double a[8]) {
    const int lane = threadIdx.x & 31;
    const bool b4 = lane & 16;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const double keep = b4 ? a[q + 4] : a[q];
        const double send = b4 ? a[q] : a[q + 4];
        a[q] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
    const bool b3 = lane & 8;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const double keep = b3 ? a[q + 2] : a[q];
        const double send = b3 ? a[q] : a[q + 2];
        a[q] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    const bool b2 = lane & 4;
    {
        const double keep = b2 ? a[1] : a[0];
        const double send = b2 ? a[0] : a[1];
        a[0] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    double v = a[0];
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    // lane l now holds value index b4*4 + b3*2 + b2 = l >> 2
    return v;
}

// Sum `cnt` slots src[i * stride + t], t < cnt, for i < nv into dst[i]
// (smem), in a fixed order; the whole CTA cooperates, 8 values per warp.
__device__ __forceinline__ void reduce_slots(const double *src, int stride, int cnt, int nv,
                                             double *dst) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int i0 = warp * 8; i0 < nv; i0 += nw * 8) {
        double a[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) a[q] = 0.0;
        for (int t = lane; t < cnt; t += 32) {
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (i0 + q < nv) a[q] += __ldcg(src + (size_t)(i0 + q) * stride + t);
        }
        const double v = warp_reduce8(a);
        const int q = lane >> 2;
        if ((lane & 3) == 0 && i0 + q < nv) dst[i0 + q] = v;
    }
}

// Write this tile's nv partial sums (smem `mine`), then reduce in two
// levels: the last tile CTA of each group of 32 tiles sums its group, the
// last group sums the group results into smem `total`.  Returns true (in
// every thread of that CTA) for the CTA holding the final sums.  Slots are
// value-major (part[i * ntiles + tile]) so the reads are coalesced.
constexpr int RGROUP = 32;
__device__ __forceinline__ bool finish_tile(const Problem &P, int tl, int nv, const double *mine,
                                            double *total) {
    __shared__ unsigned s_ticket;
    const int nt = P.ntiles;
    const int ng = (nt + RGROUP - 1) / RGROUP;
    const int g = tl / RGROUP;
    const int gcnt = min(RGROUP, nt - g * RGROUP);
    for (int i = threadIdx.x; i < nv; i += blockDim.x) P.part[(size_t)i * nt + tl] = mine[i];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_ticket = atomicAdd(P.counter + 1 + g, 1u);
    __syncthreads();
    if (s_ticket != (unsigned)(gcnt - 1)) return false;
    __threadfence();
    reduce_slots(P.part + (size_t)g * RGROUP, nt, gcnt, nv, total);
    __syncthreads();
    if (threadIdx.x == 0) P.counter[1 + g] = 0u;
    for (int i = threadIdx.x; i < nv; i += blockDim.x) P.gpart[(size_t)i * ng + g] = total[i];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_ticket = atomicAdd(P.counter, 1u);
    __syncthreads();
    if (s_ticket != (unsigned)(ng - 1)) return false;
    __threadfence();
    reduce_slots(P.gpart, ng, ng, nv, total);
    __syncthreads();
    if (threadIdx.x == 0) *P.counter = 0u;
    return true;
}

// CTA-wide sum of one value per thread (deterministic); valid in thread 0.
__device__ __forceinline__ double block_sum0(double v, double *scratch /* >= 32 */) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    v = warp_sum(v);
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < nw; ++w) s += scratch[w];
    return s;
}

// Raise a kernel's dynamic shared-memory limit.  The attribute belongs to
// the current device, so it is set once per device (a bit per device in
// `done`, per call site); devices past 63 set it on every call.
template <typename K>
inline void smem_limit_once(K *kernel, int bytes, std::atomic<unsigned long long> &done) {
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = dev < 64 ? (1ull << dev) : 0ull;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    done.fetch_or(bit, std::memory_order_release);
}

// ---- programmatic dependent launch between the kernels of a Lanczos step --
// Every step kernel waits for its predecessor at entry (griddepcontrol.wait
// returns once the previous grid has completed and its writes are visible;
// it is a no-op for a launch without the attribute) and lets its successor
// launch once its own CTAs have finished their main work, before the
// end-of-kernel reduction.  The successor's CTAs then take the SM slots of
// exiting CTAs while the last ones reduce, which hides its launch latency.
// Measured on GB300 (whole solves, in one process against the same build
// without it): 10,000 rows 81.9 -> 80.6 ms, 262,144 rows 243.1 -> 240.2 ms,
// 4.1M rows 4231 -> 4223 ms.  Triggering at kernel entry instead (4.1M-row
// solve 5.41 s -> 6.80 s) parks waiting CTAs on SM slots that multi-wave
// grids still need.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Step s of the current extension runs for this problem.
__device__ __forceinline__ bool step_active(const State *S, int s) {
    return S->status == ST_RUNNING && S->phase == PH_EXTEND && s < S->np;
}

__device__ __forceinline__ const double *step_in(const Problem &P, int j) { return (j & 1) ? P.r1 : P.r0; }
__device__ __forceinline__ double *step_out(const Problem &P, int j) { return (j & 1) ? P.r0 : P.r1; }

// ---- launch profiling (engine.cu): CUDA events around each launch ---------
enum : int { KC_SPMV = 0, KC_PROJ = 1, KC_APPLY = 2, KC_BASIS = 3, KC_RITZ = 4, KC_AUX = 5, KC_HOST = 6,
             KC_CYCLE = 7 };
void prof_begin(cudaStream_t s);
void prof_end(int cls, cudaStream_t s);

// ---- kernel entry points (kernels_step.cu / kernels_restart.cu) -----------
void launch_start_vector(const Problem *P_d, const Tile *tiles_d, int ntiles, int prob,
                         unsigned long long seed, cudaStream_t s);
void launch_norm_init(const Problem *P_d, const Tile *tiles_d, int ntiles, cudaStream_t s);
// cgs_flags: CGS_PROJ_HYBRID (hybrid projection panels), CGS_APPLY_SHADOW
// (update reads the FP32 shadow for small coefficients)
enum : int { CGS_PROJ_HYBRID = 1, CGS_APPLY_SHADOW = 2 };
void launch_step(const Problem *P_d, const Tile *tiles_d, int ntiles, const SpmvTile *stiles_d,
                 int nstiles, int step, bool fp32_any, bool external_w, int cgs_flags, const Problem *one,
                 int one_tr, cudaStream_t s);
void launch_prep_f32(const Problem *P_d, const Tile *tiles_d, int ntiles, int step, cudaStream_t s);
void launch_diag_fill(double *x, size_t count, double scale, unsigned long long key, cudaStream_t s);
void launch_cgs_kernel(const Problem *P_d, const Tile *tiles_d, int ntiles, const Problem *one, int one_tr,
                       int step, int pass, int which, bool variant, cudaStream_t s);
void launch_prep_ext(const Problem *P_d, const Tile *tiles_d, int ntiles, int step, double *xout,
                     cudaStream_t s);
void launch_restart(const Problem *P_d, int nprob, int max_ncv, cudaStream_t s);
// tensor_cores: use k_basis_tc (kernels_tc.cu) when the shape fits it.
void launch_basis(const Problem *P_d, const Tile *tiles_d, int ntiles, int max_ncv, int max_nev,
                  bool tensor_cores, cudaStream_t s);
bool basis_tc_fits(int max_ncv, int nev_max);


void launch_basis_tc(const Problem *P_d, const Tile *tiles_d, int ntiles, int nev_max, cudaStream_t s);
void launch_finalize(const Problem *P_d, int nprob, int max_ncv, cudaStream_t s);
void launch_ritz(const Problem *P_d, const Tile *tiles_d, int ntiles, int max_ncv, bool tensor_cores,
                 cudaStream_t s);
bool ritz_tc_fits(int max_ncv);
void launch_ritz_tc(const Problem *P_d, const Tile *tiles_d, int ntiles, cudaStream_t s);
void launch_spmv(const int *row_ptr, const int *col, const double *val, const Sell &sell, const SpmvTile *stiles,
                 int nstiles, const double *x, double *y, cudaStream_t s);
void launch_spmv_f32(const int *row_ptr, const int *col, const float *val, const Sell &sell, const SpmvTile *stiles,
                     int nstiles, const float *x, float *y, cudaStream_t s);
// Fill the sliced-ELL arrays (col, val, val32 may be null) of nslices
// slices from the general CSR, given ptr / len / row.
void launch_sell_fill(const int *row_ptr, const int *col, const double *val, int nslices, const long long *ptr,
                      const int *len, const int *row, int *out_col, double *out_val, float *out_val32,
                      cudaStream_t s);
void launch_gather(const Problem *P_d, int nprob, const long long *off_d, double *buf_d, cudaStream_t s);
void launch_scatter(const Problem *P_d, int nprob, const long long *off_d, const int *flag_d,
                    const double *buf_d, cudaStream_t s);
// FP64 Rayleigh-Ritz of a mixed-precision solve (kernels_refine.cu):
// G = Y^T W (part: gram_blocks(n) * k * k doubles), out = Y Z.
int gram_blocks(int n);
void launch_gram(const double *Y, const double *W, int n, int ld, int k, double *part, double *G, cudaStream_t s);
void launch_rotate(const double *Y, int n, int ld, int k, const double *Z, double *out, cudaStream_t s);
void launch_residuals(const int *row_ptr, const int *col, const double *val, int n, int k,
                      const double *values_d, const double *vectors_d, int ldv, double *out4k,
                      cudaStream_t s);

// Whole Lanczos extensions in one cooperative launch (kernels_cycle.cu):
// tiles_d holds one CycTile per CTA (problem slot, rank in its group, group
// size, rows); bars_d one barrier counter per problem slot, zeroed here;
// xpart_d nctas x 3 (MAXNCV + 2) doubles of partial sums.
int cycle_capacity();
int cycle_rows_per_cta();
struct CycTileH { int prob, rank, nb, row0, row1, pad; };
cudaError_t launch_cycle(const Problem *P_d, const void *tiles_d, int nctas, unsigned *bars_d, double *xpart_d,
                         int nprob, int steps, cudaStream_t s);

// Kernels this library launched (all host threads), and launches per
// kernel variant (HLANC_KL_*).
std::atomic<long long> &launch_counter();
std::atomic<long long> &variant_counter(int kind);

// Read-only view of a device CSR operator's arrays (engine.cu).
struct CsrView {
    int dev, nrows, ncols;
    long long nnz;
    const int *rp_d, *ci_d;
    const double *val_d;
    cudaStream_t stream;
};
int csr_view_of(hlanc_csr_t csr, CsrView *out);

}  // namespace hlanc
