// kernels_step.cu -- row-parallel kernels of one Lanczos step (HLanc.hpp:1410-1477)
//
// A step j of the reference's dsaitr is, on the device:
//   k_spmv   v_j = r / rnorm -> V[:, j];  w = A v_j            (FP64 or FP32 SpMV)
//   k_proj   h = V[:, 0:j+1]^T w  (+ ||w||^2 on the first pass)   CGS projection
//   k_apply  w -= V[:, 0:j+1] h,  ||w||^2 -> rnorm, DGKS test      CGS update
//   k_proj / k_apply again while the DGKS test (factor 0.717) asks for it.
// All decisions (second/third pass, invariant-subspace reset) are taken on
// the device by the last CTA of each kernel, so a whole restart cycle runs
// without host synchronisation and can be captured in one CUDA graph.
//
// GB300 note: these kernels stream V once per pass.  Blackwell Ultra's FP64
// rate is low, so the CGS kernels issue at most one DFMA per loaded element,
// run part of every column panel as exact fixed-point integer products on
// the integer pipes (fixed_point.cuh; launches over >= 2^18 rows), and
// accumulate every reduction in registers over a whole tile before the
// (few) shuffle additions.
#include <float.h>
#include <string.h>

#include <type_traits>

#include "internal.cuh"

namespace hlanc {

std::atomic<long long> &launch_counter() {
    static std::atomic<long long> c{0};
    return c;
}

std::atomic<long long> &variant_counter(int kind) {
    static std::atomic<long long> c[HLANC_KL_KINDS];
    return c[(kind > 0 && kind < HLANC_KL_KINDS) ? kind : 0];
}

// ---- SplitMix64 start vector (same formula as generators.start_vector) ----
__host__ __device__ inline uint64_t sm_mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__global__ void __launch_bounds__(TPB) k_start(const Problem *__restrict__ probs,
                                               const Tile *__restrict__ tiles, int prob,
                                               unsigned long long key) {
    const Tile t = tiles[blockIdx.x];
    if (t.prob != prob) return;
    const Problem &P = probs[t.prob];
    for (int r = t.row0 + threadIdx.x; r < t.row1; r += TPB) {
        uint64_t x = sm_mix(key + (uint64_t)(r + 1) * 0x9E3779B97F4A7C15ULL);
        double u = (double)(x >> 11) * 0x1.0p-53;
        P.r0[r] = 2.0 * u - 1.0;
    }
}

// rnorm = ||r0|| for problems in the initial phase (dgetv0, HLanc.hpp:1373)
__global__ void __launch_bounds__(TPB) k_norm_init(const Problem *__restrict__ probs,
                                                   const Tile *__restrict__ tiles) {
    const Tile t = tiles[blockIdx.x];
    const Problem &P = probs[t.prob];
    if (P.st->iter != -1) return;   // -1 marks "start vector written, norm pending"
    __shared__ double scratch[32], mine[1], tot[1];
    double s = 0.0;
    for (int r = t.row0 + threadIdx.x; r < t.row1; r += TPB) s = fma(P.r0[r], P.r0[r], s);
    s = block_sum0(s, scratch);
    if (threadIdx.x == 0) mine[0] = s;
    __syncthreads();
    if (!finish_tile(P, blockIdx.x - P.tile0, 1, mine, tot)) return;
    if (threadIdx.x == 0) {
        P.st->rnorm = sqrt(tot[0]);
        P.st->iter = 0;
    }
}


// ---- SpMV work units ----------------------------------------------------------------
// Short rows: thread per row, entries read directly in batches of 8 so eight
// independent gathers of x are in flight per thread; one FMA per stored entry
// and no shuffles (GB300's FP64 pipe is the scarce resource).  Measured in the
// solver on GB300 this beats staging the rows through shared memory (the
// staged form waits on its copies before the gathers can start).
constexpr int STAGE = 256;
template <typename T, typename XL, typename Emit>
__device__ __forceinline__ void spmv_short(const int *__restrict__ rp, const int *__restrict__ ci,
                                           const T *__restrict__ val, XL x, int row0,
                                           int row1, int *, T *, Emit emit) {
    for (int r = row0 + threadIdx.x; r < row1; r += TPB) {
        const int a = rp[r], b = rp[r + 1];
        T acc = T(0);
        for (int i = a; i < b; i += 8) {
            T xv[8], vv[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const bool ok = i + q < b;
                vv[q] = ok ? val[i + q] : T(0);
                xv[q] = ok ? x(ci[i + q]) : T(0);
            }
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (i + q < b) acc = fma(vv[q], xv[q], acc);
        }
        emit(r, acc);
    }
}

// Short rows of uneven length (power-law graphs): LANES lanes per row, so a
// warp waits on the longest of 32 / LANES rows instead of 32, and the lanes
// of a row read its entries contiguously; a shuffle tree sums the row.
template <typename T, int LANES, typename XL, typename Emit>
__device__ __forceinline__ void spmv_subwarp(const int *__restrict__ rp, const int *__restrict__ ci,
                                             const T *__restrict__ val, XL x, int row0,
                                             int row1, Emit emit) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int RPW = 32 / LANES;                 // rows per warp at a time
    const int q = lane & (LANES - 1);
    for (int base = row0 + warp * RPW; base < row1; base += (TPB / 32) * RPW) {
        const int r = base + lane / LANES;
        T acc = T(0);
        if (r < row1) {
            const int a = rp[r], b = rp[r + 1];
            int i = a + q;
            for (; i + LANES < b; i += 2 * LANES) {
                const T v0 = val[i], v1 = val[i + LANES];
                const T x0 = x(ci[i]), x1 = x(ci[i + LANES]);
                acc = fma(v0, x0, acc);
                acc = fma(v1, x1, acc);
            }
            if (i < b) acc = fma(val[i], x(ci[i]), acc);
        }
#pragma unroll
        for (int o = LANES / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (q == 0 && r < row1) emit(r, acc);
    }
}

// Wide row: whole CTA; the sum is valid in thread 0.
template <typename T, typename XL>
__device__ __forceinline__ T spmv_wide(const int *__restrict__ rp, const int *__restrict__ ci,
                                       const T *__restrict__ val, XL x, int r, T *red) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int a = rp[r], b = rp[r + 1];
    T acc = T(0);
#pragma unroll 4
    for (int i = a + threadIdx.x; i < b; i += TPB) acc = fma(val[i], x(ci[i]), acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __syncthreads();
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    T sum = T(0);
    if (threadIdx.x == 0)
        for (int w = 0; w < TPB / 32; ++w) sum += red[w];
    return sum;
}

// Sliced-ELL unit (kind 5): warp w takes slice s0 + w, lane l its row; the
// row's entries are summed in their CSR order (each FMA predicated on the
// row's own length, so padding adds nothing, whatever x holds), and the
// entries of four k are loaded before their FMAs.
template <typename T, typename XL, typename Emit>
__device__ __forceinline__ void spmv_slices(const Sell &S, const T *__restrict__ sval, const int *__restrict__ rp,
                                            int s0, int s1, XL x, Emit emit) {
    const int s = s0 + (int)(threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (s >= s1) return;
    const long long base = S.ptr[s];
    const int len = S.len[s];
    const int row = S.row[(size_t)s * SELL_C + lane];
    const int rl = row >= 0 ? rp[row + 1] - rp[row] : 0;
    const int *__restrict__ c = S.col + base + lane;
    const T *__restrict__ v = sval + base + lane;
    T acc = T(0);
    int k = 0;
    for (; k + 4 <= len; k += 4) {
        int cc[4];
        T vv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            cc[q] = c[(size_t)(k + q) * SELL_C];
            vv[q] = v[(size_t)(k + q) * SELL_C];
        }
        T xx[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) xx[q] = x(cc[q]);
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (k + q < rl) acc = fma(vv[q], xx[q], acc);
    }
    for (; k < len; ++k) {
        const T xv = x(c[(size_t)k * SELL_C]);
        if (k < rl) acc = fma(v[(size_t)k * SELL_C], xv, acc);
    }
    if (row >= 0) emit(row, acc);
}

// x: a functor giving x[c] (a plain load, or a conversion on the fly).
template <typename T, typename XL, typename Emit>
__device__ __forceinline__ void spmv_unit(const SpmvTile &t, const int *__restrict__ rp, const int *__restrict__ ci,
                                          const T *__restrict__ val, const Sell &sell, const T *__restrict__ sval,
                                          XL x, int *s_col, T *s_val, T *red, Emit emit) {
    if (t.kind == 5) {
        spmv_slices<T>(sell, sval, rp, t.row0, t.row1, x, emit);
    } else if (t.kind == 0) {
        spmv_short<T>(rp, ci, val, x, t.row0, t.row1, s_col, s_val, emit);
    } else if (t.kind == 3) {
        spmv_subwarp<T, 4>(rp, ci, val, x, t.row0, t.row1, emit);
    } else if (t.kind == 4) {
        spmv_subwarp<T, 8>(rp, ci, val, x, t.row0, t.row1, emit);
    } else if (t.kind == 1) {
        spmv_subwarp<T, 16>(rp, ci, val, x, t.row0, t.row1, emit);
    } else {
        const T acc = spmv_wide<T>(rp, ci, val, x, t.row0, red);
        if (threadIdx.x == 0) emit(t.row0, acc);
    }
}

template <typename T>
struct XLoad {
    const T *__restrict__ p;
    __device__ __forceinline__ T operator()(int c) const { return p[c]; }
};


// ---- SpMV of the step --------------------------------------------------------
// One CTA per SpMV unit (the hardware scheduler balances skewed units).
// v_j -> V[:, j] for the unit's rows, w = A v_j (FP64: A r, one scaling per row;
// FP32: the FP32 copy V32[:, j] that k_prep wrote).
// Six resident CTAs per SM (40 registers) keep enough gathers in flight: on
// GB300 this measured 18% faster than the unbounded 72-register build on the
// 4.1M-row Laplacian (70% of HBM standalone) and 14% faster on the power-law
// graph; streaming (evict-first) loads of the entries were slower, because
// neighbouring rows share their cache sectors.  The FP32 step kernel runs at
// 5 CTAs per SM: at 6 it spilled, and 5 measured 0.5% faster on the
// mixed-precision power-law solve.
constexpr int SPMV_CTAS_PER_SM = 6;
template <bool F32>
__global__ void __launch_bounds__(TPB, F32 ? 5 : SPMV_CTAS_PER_SM) k_spmv_step(const Problem *__restrict__ probs,
                                                   const SpmvTile *__restrict__ tiles, int ntiles, int s) {
    using T = typename std::conditional<F32, float, double>::type;
    __shared__ int s_col[(TPB / 32) * STAGE];
    __shared__ T s_val[(TPB / 32) * STAGE];
    __shared__ T red[TPB / 32];
    pdl_wait();
    const SpmvTile t = tiles[blockIdx.x];
    const Problem &P = probs[t.prob];
    const State *S = P.st;
    if ((bool)P.fp32 != F32 || P.wext || !step_active(S, s)) return;
    const int j = S->k + s;
    const double rn = S->rnorm;
    const bool scale = rn > DBL_MIN;
    const double t1 = scale ? 1.0 / rn : 1.0;
    const double *__restrict__ rin = step_in(P, j);
    double *__restrict__ w = step_out(P, j);
    double *__restrict__ vj = P.V + (size_t)j * P.ld;
    float *__restrict__ vj32 = P.V32 + (size_t)j * P.ld;
    if constexpr (F32) {
        // FP32 values and the FP32 copy of v_j (k_prep wrote V[:, j] and
        // V32[:, j] beforehand), FP32 accumulation per row.  Rounding the
        // vector once per row in k_prep, not once per gathered entry, keeps
        // conversions off GB300's narrow FP64 pipe.
        (void)vj;
        (void)vj32;
        spmv_unit<float>(t, P.row_ptr, P.col, P.val32, P.sell, P.sell.val32, XLoad<float>{vj32}, s_col, s_val, red,
                         [=](int rr, float acc) { w[rr] = (double)acc; });
    } else {
        // each row is emitted once: V[:, j] is written there too, instead of
        // in a separate pass over the unit's rows before the gathers start
        spmv_unit<double>(t, P.row_ptr, P.col, P.val, P.sell, P.sell.val, XLoad<double>{rin}, s_col, s_val, red,
                          [=](int rr, double acc) {
            const double x = rin[rr];
            const double v = scale ? x * t1 : x;
            w[rr] = scale ? acc * t1 : acc;
            vj[rr] = v;
            vj32[rr] = (float)v;
        });
    }
    pdl_trigger();
}

// v_j -> V[:, j] and V32[:, j] ahead of an FP32 SpMV (which gathers V32[:, j])
// or a host operator (xout: the staging copy of v_j).
__global__ void __launch_bounds__(TPB) k_prep(const Problem *__restrict__ probs,
                                              const Tile *__restrict__ tiles, int s, int ext,
                                              double *__restrict__ xout) {
    pdl_wait();
    const Tile t = tiles[blockIdx.x];
    const Problem &P = probs[t.prob];
    const State *S = P.st;
    if (ext ? !P.wext : !P.fp32) return;
    if (!step_active(S, s)) return;
    const int j = S->k + s;
    const double rn = S->rnorm;
    const bool scale = rn > DBL_MIN;
    const double t1 = scale ? 1.0 / rn : 1.0;
    const double *__restrict__ rin = step_in(P, j);
    double *__restrict__ vj = P.V + (size_t)j * P.ld;
    float *__restrict__ vj32 = P.V32 + (size_t)j * P.ld;
    for (int r = t.row0 + threadIdx.x; r < t.row1; r += TPB) {
        const double x = rin[r];
        const double v = scale ? x * t1 : x;
        vj[r] = v;
        vj32[r] = (float)v;
        if (ext) xout[r] = v;
    }
}

// ---- CGS projection: h = V[:, 0:c)^T w  (+ ||w||^2 on pass 1) ----------------
// Thread per row, columns in panels (16 wide for the FP64 kernel, 8 for the
// hybrid one): each thread keeps one accumulator per panel column for all
// the rows it visits in the tile (coalesced column reads), then one
// transposed warp reduction per panel.  Panel shapes are template parameters
// picked from the device-known column count, so no instruction is issued
// for an absent column (predicated-off FP64 instructions still occupy
// GB300's FP64 pipe).
//
// The hybrid kernel (HY) splits a full panel into 5 FP64 columns (one DFMA
// per element) and 3 integer columns (exact fixed-point products, fx_*),
// which keeps the FP64 and the integer pipes busy at once.  Measured on
// GB300 (n = 4.1M rows, 32 columns, HBM-resident V): 176 us against 254 us
// for all-FP64 panels (8- or 16-wide), i.e. 5.9 against 4.1 TB/s; 4+4 was
// equal, 3+5, 2+6 and 6+6 splits and 3, 5 or 6 CTAs per SM were slower.
// w's fixed-point scale is the largest exponent of the thread's own rows on
// pass 1 (one extra read of w, which also gives ||w||^2) and 2 ||w|| on
// later passes (||w|| is known from the previous k_apply).
// Warp sums of every panel go to wsum[warp * WSTRIDE + column] without a
// barrier; one cross-warp sum after the last panel (proj_combine).  Measured
// on GB300: a cross-warp reduction with two barriers per panel left every
// warp waiting for the slowest at each panel boundary.
constexpr int WSTRIDE = MAXNCV + 1;

template <int ND, int NI, bool with_norm = false>
__device__ __forceinline__ void proj_panel(const double *__restrict__ V, size_t ld, int row0, int row1,
                                           const double *__restrict__ w, int c0, int ew, double *wsum) {
    constexpr int NC = ND + NI;
    constexpr int NA = (NC + 7) / 8 * 8;
    static_assert(NC >= 1 && NC <= 16 && (NI == 0 || NC <= 8), "panel width");
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double acc[NA];
#pragma unroll
    for (int i = 0; i < NA; ++i) acc[i] = 0.0;
    FxAcc A[NI > 0 ? NI : 1];
#pragma unroll
    for (int i = 0; i < NI; ++i) fx_zero(A[i]);
    const int rsw = 1027 + ew;
    double nrm = 0.0;
    int steps = 0;
    const double *__restrict__ vc = V + (size_t)c0 * ld;
    for (int r = row0 + (int)threadIdx.x; r < row1; r += TPB) {
        const double wr = w[r];
        if constexpr (with_norm) nrm = fma(wr, wr, nrm);
        const double *__restrict__ vr = vc + r;
#pragma unroll
        for (int k = 0; k < ND; ++k) acc[k] = fma(__ldcs(vr + (size_t)k * ld), wr, acc[k]);
        if constexpr (NI > 0) {
            int w1, w0;
            fx_split(wr, rsw, w1, w0);
#pragma unroll
            for (int k = 0; k < NI; ++k) {
                int v1, v0;
                fx_split(__ldcs(vr + (size_t)(ND + k) * ld), FX_RS_UNIT, v1, v0);
                fx_mac(A[k], v1, v0, w1, w0);
            }
            if (++steps == FX_MACS) {
                steps = 0;
#pragma unroll
                for (int k = 0; k < NI; ++k) fx_carry(A[k]);
            }
        }
    }
    // products carry the scales 2^57 (V) and 2^(57 - ew) (w)
#pragma unroll
    for (int k = 0; k < NI; ++k) acc[ND + k] = fx_to_double(A[k], ew - 114);
    // lane l holds, per group g of 8 columns, the warp sum of column 8g + (l >> 2)
    double *ws = wsum + warp * WSTRIDE + c0;
#pragma unroll
    for (int g = 0; g < NA / 8; ++g) {
        const double v = warp_reduce8(acc + 8 * g);
        const int q = 8 * g + (lane >> 2);
        if ((lane & 3) == 0 && q < NC) ws[q] = v;
    }
    if constexpr (with_norm) {
        nrm = warp_sum(nrm);
        if (lane == 0) ws[NC] = nrm;
    }
}

// red[i] = sum over the warps of wsum[warp][i], i < nv, in warp order
__device__ __forceinline__ void proj_combine(const double *wsum, int nv, double *red) {
    __syncthreads();
    for (int i = threadIdx.x; i < nv; i += TPB) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < TPB / 32; ++q) s += wsum[q * WSTRIDE + i];
        red[i] = s;
    }
    __syncthreads();
}

template <bool NORM>
__device__ __forceinline__ void proj_panel_fp64(const double *__restrict__ V, size_t ld, int row0, int row1,
                                                const double *__restrict__ w, int c0, int cc, double *wsum) {
    switch (cc) {
    case 1: proj_panel<1, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    case 2: proj_panel<2, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    case 3: proj_panel<3, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    case 4: proj_panel<4, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    case 5: proj_panel<5, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    case 6: proj_panel<6, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    case 7: proj_panel<7, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    case 8: proj_panel<8, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    case 9: proj_panel<9, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    case 10: proj_panel<10, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    case 11: proj_panel<11, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    case 12: proj_panel<12, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    case 13: proj_panel<13, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    case 14: proj_panel<14, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    default: proj_panel<15, 0, NORM>(V, ld, row0, row1, w, c0, 0, wsum); break;
    }
}

__device__ __forceinline__ void proj_panel_hybrid(const double *__restrict__ V, size_t ld, int row0, int row1,
                                                  const double *__restrict__ w, int c0, int cc, int ew,
                                                  double *wsum) {
    switch (cc) {
    case 1: proj_panel<1, 0>(V, ld, row0, row1, w, c0, ew, wsum); break;
    case 2: proj_panel<1, 1>(V, ld, row0, row1, w, c0, ew, wsum); break;
    case 3: proj_panel<2, 1>(V, ld, row0, row1, w, c0, ew, wsum); break;
    case 4: proj_panel<2, 2>(V, ld, row0, row1, w, c0, ew, wsum); break;
    case 5: proj_panel<3, 2>(V, ld, row0, row1, w, c0, ew, wsum); break;
    case 6: proj_panel<3, 3>(V, ld, row0, row1, w, c0, ew, wsum); break;
    default: proj_panel<4, 3>(V, ld, row0, row1, w, c0, ew, wsum); break;
    }
}

// ONE: a launch over a single problem, whose descriptor is passed by value
// (kernel parameter space, so the basis pointer and stride stay in uniform
// registers) with tiles of tr rows in blockIdx order.  Measured on GB300
// (4.1M rows, 32 columns): 207 us against 218 us for descriptor and tile
// loads from the tables, which batched launches need.
template <bool ONE>
struct TileRows {
    int row0, row1, prob;
    __device__ __forceinline__ TileRows(const Tile *__restrict__ tiles, const Problem &P1, int tr) {
        if constexpr (ONE) {
            row0 = blockIdx.x * tr;
            row1 = min(P1.n, row0 + tr);
            prob = 0;
        } else {
            const Tile t = tiles[blockIdx.x];
            row0 = t.row0;
            row1 = t.row1;
            prob = t.prob;
        }
    }
};

template <bool HY, bool ONE>
__global__ void __launch_bounds__(TPB, 4) k_proj(const Problem *__restrict__ probs,
                                              const Tile *__restrict__ tiles, const Problem P1, int tr,
                                              int s, int pass) {
    pdl_wait();
    const TileRows<ONE> t(tiles, P1, tr);
    const Problem &P = ONE ? P1 : probs[t.prob];
    State *S = P.st;
    if (!step_active(S, s)) return;
    if ((pass == 2 && !S->need2) || (pass == 3 && !S->need3)) return;
    const int j = S->k + s;
    const int c = j + 1;
    const int m = P.ncv;
    const double *__restrict__ w = step_out(P, j);
    const double *__restrict__ V = P.V;
    const size_t ld = (size_t)P.ld;
    __shared__ double red[MAXNCV + 1], tot[MAXNCV + 1];
    __shared__ double sm[32];
    __shared__ double wsum[(TPB / 32) * WSTRIDE];
    if constexpr (HY) {
        int ew;
        if (pass == 1) {
            // ||w||^2 and the scale of this thread's rows (HLanc.hpp:1429)
            unsigned mx = 0;
            double nrm = 0.0;
            for (int r = t.row0 + threadIdx.x; r < t.row1; r += TPB) {
                const double x = w[r];
                nrm = fma(x, x, nrm);
                mx = max(mx, fx_hi_abs(x));
            }
            ew = fx_scale(mx);
            nrm = block_sum0(nrm, sm);
            if (threadIdx.x == 0) red[c] = nrm;
            __syncthreads();
        } else {
            ew = fx_scale(fx_hi_abs(S->rnorm)) + 1;   // |w_i| <= ||w|| < 2^(ew + 1)
        }
        // full panels called directly (a switch around every panel measured
        // 5% slower), then the remainder
        int c0 = 0;
        for (; c0 + 8 <= c; c0 += 8) proj_panel<5, 3>(V, ld, t.row0, t.row1, w, c0, ew, wsum);
        if (c0 < c) proj_panel_hybrid(V, ld, t.row0, t.row1, w, c0, c - c0, ew, wsum);
        pdl_trigger();
        proj_combine(wsum, c, red);        // red[c] (pass 1) came from the scan
    } else {
        // 16-column panels (measured fastest for the FP64 kernel: 64
        // registers, 4 CTAs per SM); ||w||^2 rides with the last panel on pass 1
        int c0 = 0;
        for (; c0 + 16 <= c; c0 += 16) {
            if (pass == 1 && c0 + 16 == c) proj_panel<16, 0, true>(V, ld, t.row0, t.row1, w, c0, 0, wsum);
            else proj_panel<16, 0>(V, ld, t.row0, t.row1, w, c0, 0, wsum);
        }
        if (c0 < c) {
            if (pass == 1) proj_panel_fp64<true>(V, ld, t.row0, t.row1, w, c0, c - c0, wsum);
            else proj_panel_fp64<false>(V, ld, t.row0, t.row1, w, c0, c - c0, wsum);
        }
        pdl_trigger();
        proj_combine(wsum, c + (pass == 1 ? 1 : 0), red);
    }
    __syncthreads();
    if (!finish_tile(P, blockIdx.x - P.tile0, c + (pass == 1 ? 1 : 0), red, tot)) return;
    double *h = P.small + SM_H(m);
    double *hv = P.small + SM_HV(m);
    for (int i = threadIdx.x; i < c; i += TPB) hv[i] = tot[i];
    if (threadIdx.x == 0) {
        if (pass == 1) {
            h[m + j] = tot[j];                       // alpha_j, HLanc.hpp:1433
            h[j] = (j == 0) ? 0.0 : S->rnorm;         // beta_j,  HLanc.hpp:1434-1438
            S->wnorm = sqrt(tot[c]);                  // HLanc.hpp:1429
            S->spmv += 1;
        } else {
            h[m + j] += tot[j];                       // HLanc.hpp:1447
        }
        S->passes += 1;
    }
}

// ---- CGS update: w -= V[:, 0:c) h ; DGKS decision ------------------------------
// SHADOW (the default update): a column whose coefficient is tiny next to
// the norm s of the vector being updated, |h_i| <= 2^-32 s / c, is read from
// the FP32 shadow V32 and accumulated in FP32; the other columns read V and
// accumulate in FP64.  In a Lanczos step only v_j and v_{j-1} carry large
// coefficients (alpha_j, beta_j) on the first pass; the older columns' are
// at the level of the basis' loss of orthogonality, and on the second pass
// every coefficient is.  The FP32 terms' error, relative (c + 3) 2^-24 each,
// sums to at most (c + 3) 2^-56 s: the FP64 rounding level of the update
// (the reference's FP64 gemv has a worst case of c 2^-53 |V||h|).  So the
// update keeps FP64 accuracy while most columns move 4 bytes per element
// instead of 8, and only the FP64 columns use the (slow on GB300) FP64 pipe.
// s is ||w|| on the first pass (from the projection) and the norm left by
// the previous update on later passes; the FP32 coefficients are scaled by
// 2^-ilogb(s) so no value approaches FP32's range limits.  A non-finite or
// zero s sends every column to FP64.  Without SHADOW (HLANC_CGS_FP64) every
// column is an FP64 FMA.
// The last R < 8 columns of an update, for two consecutive rows, unrolled
// so that their loads are issued together.
template <int R>
__device__ __forceinline__ void apply_tail_fp64(const double *__restrict__ vr, size_t ld, int k,
                                                const double *hs, double2 &acc) {
    double2 v[R > 0 ? R : 1];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = __ldcs(reinterpret_cast<const double2 *>(vr + (size_t)(k + q) * ld));
#pragma unroll
    for (int q = 0; q < R; ++q) {
        acc.x = fma(-v[q].x, hs[k + q], acc.x);
        acc.y = fma(-v[q].y, hs[k + q], acc.y);
    }
}

__device__ __forceinline__ void apply_tail_fp64_n(const double *__restrict__ vr, size_t ld, int k, int r,
                                                  const double *hs, double2 &acc) {
    switch (r) {
    case 1: apply_tail_fp64<1>(vr, ld, k, hs, acc); break;
    case 2: apply_tail_fp64<2>(vr, ld, k, hs, acc); break;
    case 3: apply_tail_fp64<3>(vr, ld, k, hs, acc); break;
    case 4: apply_tail_fp64<4>(vr, ld, k, hs, acc); break;
    case 5: apply_tail_fp64<5>(vr, ld, k, hs, acc); break;
    case 6: apply_tail_fp64<6>(vr, ld, k, hs, acc); break;
    case 7: apply_tail_fp64<7>(vr, ld, k, hs, acc); break;
    default: break;
    }
}

template <int R>
__device__ __forceinline__ void apply_tail_f32(const float *__restrict__ vr, size_t ld, int k, const float *hs,
                                               float2 &acc) {
    float2 v[R > 0 ? R : 1];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = __ldcs(reinterpret_cast<const float2 *>(vr + (size_t)(k + q) * ld));
#pragma unroll
    for (int q = 0; q < R; ++q) {
        acc.x = fmaf(v[q].x, hs[k + q], acc.x);
        acc.y = fmaf(v[q].y, hs[k + q], acc.y);
    }
}

__device__ __forceinline__ void apply_tail_f32_n(const float *__restrict__ vr, size_t ld, int k, int r,
                                                 const float *hs, float2 &acc) {
    switch (r) {
    case 1: apply_tail_f32<1>(vr, ld, k, hs, acc); break;
    case 2: apply_tail_f32<2>(vr, ld, k, hs, acc); break;
    case 3: apply_tail_f32<3>(vr, ld, k, hs, acc); break;
    case 4: apply_tail_f32<4>(vr, ld, k, hs, acc); break;
    case 5: apply_tail_f32<5>(vr, ld, k, hs, acc); break;
    case 6: apply_tail_f32<6>(vr, ld, k, hs, acc); break;
    case 7: apply_tail_f32<7>(vr, ld, k, hs, acc); break;
    default: break;
    }
}

// Six CTAs per SM for single-problem launches (40 registers); the batched
// form's table loads need a few more registers, so it runs five.
template <bool SHADOW, bool ONE>
__global__ void __launch_bounds__(TPB, ONE ? 6 : 5) k_apply(const Problem *__restrict__ probs,
                                                  const Tile *__restrict__ tiles, const Problem P1, int tr,
                                                  int s, int pass) {
    pdl_wait();
    const TileRows<ONE> t(tiles, P1, tr);
    const Problem &P = ONE ? P1 : probs[t.prob];
    State *S = P.st;
    if (!step_active(S, s)) return;
    if ((pass == 2 && !S->need2) || (pass == 3 && !S->need3)) return;
    const int j = S->k + s;
    const int c = j + 1;
    const int m = P.ncv;
    double *__restrict__ w = step_out(P, j);
    __shared__ double hs[MAXNCV];
    __shared__ float h32s[MAXNCV];
    __shared__ double scratch[32], mine[1], tot[1];
    __shared__ int s_zero, s_t;
    const double *hv = P.small + SM_HV(m);
    // norm of the vector this pass updates (HLanc.hpp:1429 / 1440-1458)
    const double sc = pass == 1 ? S->wnorm : S->rnorm;
    const bool usable = SHADOW && sc > 0.0 && sc <= DBL_MAX;
    const double thr = usable ? ldexp(sc, -32) / c : 0.0;
    if (threadIdx.x == 0) s_t = usable ? c : 0;
    __syncthreads();
    for (int i = threadIdx.x; i < c; i += TPB) {
        const double h = hv[i];
        hs[i] = h;
        if (usable && !(fabs(h) <= thr)) atomicMin(&s_t, i);
    }
    __syncthreads();
    const int tf = s_t;                       // columns [0, tf) in FP32, [tf, c) in FP64
    const int ke = usable ? -ilogb(sc) : 0;
    for (int i = threadIdx.x; i < tf; i += TPB) h32s[i] = (float)ldexp(hs[i], ke);
    __syncthreads();
    const double unscale = ldexp(1.0, -ke);
    const size_t ld = (size_t)P.ld;
    double nrm = 0.0;
    // Two consecutive rows per thread (8-byte FP32 / 16-byte FP64 loads):
    // twice the bytes in flight per load.  Tiles start on 64-row boundaries;
    // an odd last row n - 1 is paired with padding row n (< ld), whose w and
    // V entries are zero and stay zero, so it adds nothing.
    const int rend = min(P.ld, (t.row1 + 1) & ~1);
    for (int r = t.row0 + 2 * (int)threadIdx.x; r < rend; r += 2 * TPB) {
        double2 acc = *reinterpret_cast<const double2 *>(w + r);
        int k = 0;
        if (SHADOW && tf > 0) {
            const float *__restrict__ vr32 = P.V32 + r;
            float2 a32 = make_float2(0.0f, 0.0f);
            for (; k + 8 <= tf; k += 8) {
                float2 v[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) v[q] = __ldcs(reinterpret_cast<const float2 *>(vr32 + (size_t)(k + q) * ld));
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    a32.x = fmaf(v[q].x, h32s[k + q], a32.x);
                    a32.y = fmaf(v[q].y, h32s[k + q], a32.y);
                }
            }
            apply_tail_f32_n(vr32, ld, k, tf - k, h32s, a32);
            k = tf;
            acc.x = fma(-(double)a32.x, unscale, acc.x);
            acc.y = fma(-(double)a32.y, unscale, acc.y);
        }
        const double *__restrict__ vr = P.V + r;
        for (; k + 8 <= c; k += 8) {
            double2 v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = __ldcs(reinterpret_cast<const double2 *>(vr + (size_t)(k + q) * ld));
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                acc.x = fma(-v[q].x, hs[k + q], acc.x);
                acc.y = fma(-v[q].y, hs[k + q], acc.y);
            }
        }
        apply_tail_fp64_n(vr, ld, k, c - k, hs, acc);
        *reinterpret_cast<double2 *>(w + r) = acc;
        nrm = fma(acc.x, acc.x, nrm);
        nrm = fma(acc.y, acc.y, nrm);
    }
    pdl_trigger();
    nrm = block_sum0(nrm, scratch);
    if (threadIdx.x == 0) mine[0] = nrm;
    __syncthreads();
    if (!finish_tile(P, blockIdx.x - P.tile0, 1, mine, tot)) return;
    if (threadIdx.x == 0) {
        const double nr = sqrt(tot[0]);
        s_zero = 0;
        S->sumc += c;
        S->sumt += tf;
        if (pass == 1) {                               // HLanc.hpp:1440-1444
            S->rnorm = nr;
            S->need2 = nr < S->wnorm * 0.717;
            S->need3 = 0;
        } else if (pass == 2) {                        // HLanc.hpp:1450-1458
            S->need3 = !(nr > S->rnorm * 0.717);
            S->rnorm = nr;
        } else {                                       // HLanc.hpp:1450-1463
            if (nr > S->rnorm * 0.717) {
                S->rnorm = nr;
            } else {
                S->rnorm = 0.0;
                s_zero = 1;
            }
        }
    }
    __syncthreads();
    if (s_zero)   // invariant subspace: resid = 0 (rare; one CTA clears the vector)
        for (int r = threadIdx.x; r < P.n; r += TPB) w[r] = 0.0;
}

// ---- standalone SpMV (operator() of dcsrmv_operator_gpu) -------------------
template <typename T>
__global__ void __launch_bounds__(TPB, SPMV_CTAS_PER_SM) k_spmv_plain(const int *__restrict__ rp,
                                                    const int *__restrict__ ci,
                                                    const T *__restrict__ val, const Sell sell,
                                                    const T *__restrict__ sval,
                                                    const SpmvTile *__restrict__ tiles, int ntiles,
                                                    const T *__restrict__ x, T *__restrict__ y) {
    __shared__ int s_col[(TPB / 32) * STAGE];
    __shared__ T s_val[(TPB / 32) * STAGE];
    __shared__ T red[TPB / 32];
    for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x)
        spmv_unit<T>(tiles[ti], rp, ci, val, sell, sval, XLoad<T>{x}, s_col, s_val, red,
                     [=](int rr, T acc) { y[rr] = acc; });
}

// ---- residuals of k Ritz pairs (demo/verify_eigs.cu:52-98) ------------------
// out4k[4*i + 0] = ||A v - lambda v||^2, +1 = max|Av - lambda v|, +2 = max|Av|, +3 = max|lambda v|
__global__ void __launch_bounds__(TPB) k_residuals(const int *__restrict__ rp,
                                                   const int *__restrict__ ci,
                                                   const double *__restrict__ val, int n,
                                                   const double *__restrict__ values,
                                                   const double *__restrict__ V, int ldv,
                                                   double *__restrict__ part) {
    const int i = blockIdx.y;
    const double lam = values[i];
    const double *v = V + (size_t)i * ldv;
    double ss = 0.0, md = 0.0, ma = 0.0, mb = 0.0;
    for (int r = blockIdx.x * TPB + threadIdx.x; r < n; r += gridDim.x * TPB) {
        double acc = 0.0;
        for (int q = rp[r]; q < rp[r + 1]; ++q) acc = fma(val[q], v[ci[q]], acc);
        const double lv = lam * v[r];
        const double d = acc - lv;
        ss = fma(d, d, ss);
        md = fmax(md, fabs(d));
        ma = fmax(ma, fabs(acc));
        mb = fmax(mb, fabs(lv));
    }
    __shared__ double sh[4][TPB / 32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    ss = warp_sum(ss);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        md = fmax(md, __shfl_xor_sync(0xffffffffu, md, o));
        ma = fmax(ma, __shfl_xor_sync(0xffffffffu, ma, o));
        mb = fmax(mb, __shfl_xor_sync(0xffffffffu, mb, o));
    }
    if (lane == 0) { sh[0][warp] = ss; sh[1][warp] = md; sh[2][warp] = ma; sh[3][warp] = mb; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0, c = 0, d = 0;
        for (int q = 0; q < TPB / 32; ++q) { a += sh[0][q]; b = fmax(b, sh[1][q]); c = fmax(c, sh[2][q]); d = fmax(d, sh[3][q]); }
        double *o = part + ((size_t)i * gridDim.x + blockIdx.x) * 4;
        o[0] = a; o[1] = b; o[2] = c; o[3] = d;
    }
}

__global__ void k_residuals_final(const double *__restrict__ part, int nblk, int k,
                                  double *__restrict__ out4k) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k) return;
    double a = 0, b = 0, c = 0, d = 0;
    for (int q = 0; q < nblk; ++q) {
        const double *o = part + ((size_t)i * nblk + q) * 4;
        a += o[0]; b = fmax(b, o[1]); c = fmax(c, o[2]); d = fmax(d, o[3]);
    }
    out4k[4 * i + 0] = a; out4k[4 * i + 1] = b; out4k[4 * i + 2] = c; out4k[4 * i + 3] = d;
}

// ---- launchers --------------------------------------------------------------
static int spmv_grid(int nstiles) { return nstiles > 0 ? nstiles : 1; }

void launch_start_vector(const Problem *P_d, const Tile *tiles_d, int ntiles, int prob,
                         unsigned long long seed, cudaStream_t s) {
    const unsigned long long key = sm_mix(seed * 0xD1B54A32D192ED03ULL + 0ULL);
    prof_begin(s);
    k_start<<<ntiles, TPB, 0, s>>>(P_d, tiles_d, prob, key);
    prof_end(KC_AUX, s);
    launch_counter() += 1;
}

void launch_norm_init(const Problem *P_d, const Tile *tiles_d, int ntiles, cudaStream_t s) {
    prof_begin(s);
    k_norm_init<<<ntiles, TPB, 0, s>>>(P_d, tiles_d);
    prof_end(KC_AUX, s);
    launch_counter() += 1;
}

void launch_prep_f32(const Problem *P_d, const Tile *tiles_d, int ntiles, int step, cudaStream_t s) {
    prof_begin(s);
    k_prep<<<ntiles, TPB, 0, s>>>(P_d, tiles_d, step, 0, nullptr);
    prof_end(KC_SPMV, s);
    launch_counter() += 1;
}

void launch_prep_ext(const Problem *P_d, const Tile *tiles_d, int ntiles, int step, double *xout,
                     cudaStream_t s) {
    prof_begin(s);
    k_prep<<<ntiles, TPB, 0, s>>>(P_d, tiles_d, step, 1, xout);
    prof_end(KC_AUX, s);
    launch_counter() += 1;
}

// One Lanczos step for every active problem of the tile table.  With
// external_w the operator output was already written by the host path.
void launch_step(const Problem *P_d, const Tile *tiles_d, int ntiles, const SpmvTile *stiles_d,
                 int nstiles, int step, bool fp32_any, bool external_w, int cgs_flags, const Problem *one,
                 int one_tr, cudaStream_t s) {
    if (!external_w) {
        if (fp32_any) {
            prof_begin(s);
            (void)launch_pdl(k_prep, dim3(ntiles), dim3(TPB), s, P_d, tiles_d, step, 0, (double *)nullptr);
            prof_end(KC_SPMV, s);
            prof_begin(s);
            (void)launch_pdl(k_spmv_step<true>, dim3(spmv_grid(nstiles)), dim3(TPB), s, P_d, stiles_d, nstiles, step);
            prof_end(KC_SPMV, s);
            launch_counter() += 2;
        }
        prof_begin(s);
        (void)launch_pdl(k_spmv_step<false>, dim3(spmv_grid(nstiles)), dim3(TPB), s, P_d, stiles_d, nstiles, step);
        prof_end(KC_SPMV, s);
        launch_counter() += 1;
    }
    for (int pass = 1; pass <= 3; ++pass) {
        prof_begin(s);
        launch_cgs_kernel(P_d, tiles_d, ntiles, one, one_tr, step, pass, 0, (cgs_flags & CGS_PROJ_HYBRID) != 0, s);
        prof_end(KC_PROJ, s);
        prof_begin(s);
        launch_cgs_kernel(P_d, tiles_d, ntiles, one, one_tr, step, pass, 1, (cgs_flags & CGS_APPLY_SHADOW) != 0, s);
        prof_end(KC_APPLY, s);
    }
}

// ---- diagnostics: one CGS kernel alone (hlanc_diag_cgs) -----------------------
__global__ void k_diag_fill(double *__restrict__ x, size_t count, double scale, unsigned long long key) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        const uint64_t z = sm_mix(key + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ULL);
        x[i] = scale * (2.0 * ((double)(z >> 11) * 0x1.0p-53) - 1.0);
    }
}

void launch_diag_fill(double *x, size_t count, double scale, unsigned long long key, cudaStream_t s) {
    k_diag_fill<<<1216, 256, 0, s>>>(x, count, scale, key);
    launch_counter() += 1;
}

// which: 0 = projection (variant: hybrid FP64 + fixed-point panels), 1 =
// update (variant: FP32 shadow for small coefficients).  one: the host copy
// of the descriptor of a single-problem launch (tiles of one_tr rows), or null.
void launch_cgs_kernel(const Problem *P_d, const Tile *tiles_d, int ntiles, const Problem *one, int one_tr,
                       int step, int pass, int which, bool variant, cudaStream_t s) {
    Problem P1;
    if (one) P1 = *one;
    else memset(&P1, 0, sizeof P1);
    const int code = (which << 2) | (variant ? 2 : 0) | (one ? 1 : 0);
    variant_counter(which == 0 ? (variant ? HLANC_KL_PROJ_HYBRID : HLANC_KL_PROJ_FP64)
                               : (variant ? HLANC_KL_APPLY_SHADOW : HLANC_KL_APPLY_FP64)) += 1;
    const dim3 g(ntiles), b(TPB);
    switch (code) {
    case 0: (void)launch_pdl(k_proj<false, false>, g, b, s, P_d, tiles_d, P1, one_tr, step, pass); break;
    case 1: (void)launch_pdl(k_proj<false, true>, g, b, s, P_d, tiles_d, P1, one_tr, step, pass); break;
    case 2: (void)launch_pdl(k_proj<true, false>, g, b, s, P_d, tiles_d, P1, one_tr, step, pass); break;
    case 3: (void)launch_pdl(k_proj<true, true>, g, b, s, P_d, tiles_d, P1, one_tr, step, pass); break;
    case 4: (void)launch_pdl(k_apply<false, false>, g, b, s, P_d, tiles_d, P1, one_tr, step, pass); break;
    case 5: (void)launch_pdl(k_apply<false, true>, g, b, s, P_d, tiles_d, P1, one_tr, step, pass); break;
    case 6: (void)launch_pdl(k_apply<true, false>, g, b, s, P_d, tiles_d, P1, one_tr, step, pass); break;
    default: (void)launch_pdl(k_apply<true, true>, g, b, s, P_d, tiles_d, P1, one_tr, step, pass); break;
    }
    launch_counter() += 1;
}

void launch_spmv(const int *row_ptr, const int *col, const double *val, const Sell &sell, const SpmvTile *stiles,
                 int nstiles, const double *x, double *y, cudaStream_t s) {
    if (nstiles <= 0) return;
    k_spmv_plain<double><<<spmv_grid(nstiles), TPB, 0, s>>>(row_ptr, col, val, sell, sell.val, stiles, nstiles, x, y);
    launch_counter() += 1;
}

void launch_spmv_f32(const int *row_ptr, const int *col, const float *val, const Sell &sell, const SpmvTile *stiles,
                     int nstiles, const float *x, float *y, cudaStream_t s) {
    if (nstiles <= 0) return;
    k_spmv_plain<float><<<spmv_grid(nstiles), TPB, 0, s>>>(row_ptr, col, val, sell, sell.val32, stiles, nstiles, x, y);
    launch_counter() += 1;
}

// Sliced-ELL fill: thread (slice, lane) copies its row's entries to
// positions ptr[s] + k * SELL_C + lane (coalesced writes across the warp)
// and pads the slice's remaining k with column 0, value 0.
__global__ void __launch_bounds__(TPB) k_sell_fill(const int *__restrict__ rp, const int *__restrict__ ci,
                                                   const double *__restrict__ va, int nslices,
                                                   const long long *__restrict__ ptr, const int *__restrict__ len,
                                                   const int *__restrict__ row, int *__restrict__ oc,
                                                   double *__restrict__ ov, float *__restrict__ ov32) {
    const long long gid = (long long)blockIdx.x * TPB + threadIdx.x;
    const int s = (int)(gid / SELL_C), lane = (int)(gid % SELL_C);
    if (s >= nslices) return;
    const int r = row[(size_t)s * SELL_C + lane];
    const int a = r >= 0 ? rp[r] : 0, rl = r >= 0 ? rp[r + 1] - a : 0;
    const long long base = ptr[s] + lane;
    for (int k = 0; k < len[s]; ++k) {
        const long long o = base + (long long)k * SELL_C;
        const bool in = k < rl;
        const double v = in ? va[a + k] : 0.0;
        if (oc) oc[o] = in ? ci[a + k] : 0;
        if (ov) ov[o] = v;
        if (ov32) ov32[o] = (float)v;
    }
}

void launch_sell_fill(const int *row_ptr, const int *col, const double *val, int nslices, const long long *ptr,
                      const int *len, const int *row, int *out_col, double *out_val, float *out_val32,
                      cudaStream_t s) {
    if (nslices <= 0) return;
    const long long threads = (long long)nslices * SELL_C;
    k_sell_fill<<<(unsigned)((threads + TPB - 1) / TPB), TPB, 0, s>>>(row_ptr, col, val, nslices, ptr, len, row,
                                                                    out_col, out_val, out_val32);
    launch_counter() += 1;
}

void launch_residuals(const int *row_ptr, const int *col, const double *val, int n, int k,
                      const double *values_d, const double *vectors_d, int ldv, double *out4k,
                      cudaStream_t s) {
    int nblk = (n + TPB - 1) / TPB;
    if (nblk > 304) nblk = 304;
    if (nblk < 1) nblk = 1;
    double *part = nullptr;
    cudaMallocAsync(&part, sizeof(double) * 4 * (size_t)nblk * (size_t)k, s);
    k_residuals<<<dim3(nblk, k), TPB, 0, s>>>(row_ptr, col, val, n, values_d, vectors_d, ldv, part);
    k_residuals_final<<<(k + 127) / 128, 128, 0, s>>>(part, nblk, k, out4k);
    cudaFreeAsync(part, s);
    launch_counter() += 2;
}

}  // namespace hlanc
