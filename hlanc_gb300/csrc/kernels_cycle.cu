// kernels_cycle.cu -- a whole Lanczos extension (dsaitr, HLanc.hpp:1404-1482)
// in one cooperative launch, for problems too small to fill the GPU.
//
// A small solve (the 10,000-row Laplacian: 50k entries, 30 basis columns)
// is latency-bound when every Lanczos step is seven launches: each launch
// and its end-of-kernel reduction cost several microseconds of an almost
// idle GPU.  Here every CTA of a problem's group owns a row range for the
// whole extension and the step's phases are separated by group barriers:
//
//   SpMV of own rows (w = A r / rnorm, V[:, j] and its FP32 copy)
//   CGS projection partials  -> barrier -> every CTA sums all partials
//   CGS update of own rows, then the second pass's projection partials of
//   the updated rows with its norm -> barrier -> every CTA sums them
//   (DGKS: second update -> barrier -> norm; a rare third pass as before)
//
// Three group barriers per step instead of four: the second projection
// needs only own rows of the updated vector, so it shares the barrier that
// the first update's norm needs (2-D Laplacian 10,000 rows: 61.7 -> 53.3 ms
// per solve).  Results are bitwise those of the four-barrier order: every
// partial is summed over the same rows in the same order.
//
// Every CTA reduces the partials itself, in the same order, so all CTAs
// hold bitwise-identical h, norms and DGKS decisions without another
// exchange; the group's rank-0 CTA writes them to the problem's State for
// the host.  Partials of a projection and of an update live in different
// slots, so no CTA overwrites a slot another is still reading.
//
// The launch is cooperative (all CTAs co-resident, a documented guarantee),
// and every barrier wait is bounded: a wait that gives up sets State::err,
// and CTAs still waiting see it and return, so the kernel always ends.
// Several problems may share the launch (a batch or a serving lane), each
// with its own CTA group and barrier counter; groups never wait on each
// other.
#include <float.h>

#include "internal.cuh"

namespace hlanc {

constexpr int CTPB = 128;                  // threads (= rows per pass) of a CTA

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Group barrier: returns false (in every thread of the CTA) when the wait
// gave up or another CTA of the group reported an error.
__device__ __forceinline__ bool group_sync(unsigned *bar, unsigned nb, unsigned &target, unsigned limit,
                                           State *S, int *s_ok) {
    __syncthreads();
    target += nb;
    if (threadIdx.x == 0) {
        int ok = 1;
        __threadfence();   // this CTA's partials (written before the __syncthreads) before its arrival
        atomicAdd(bar, 1u);
        // The acquire loads order this CTA's later reads after the other
        // CTAs' arrivals (and so after their fenced partials); the poll
        // spins without sleeping, since a barrier is on the critical path
        // of every Lanczos step.
        for (unsigned spins = 0;; ++spins) {
            if (ld_acquire(bar) >= target) break;
            if (*(volatile int *)&S->err != DEV_ERR_NONE) { ok = 0; break; }
            if (spins >= limit) {
                atomicExch(&S->err, DEV_ERR_GRID_WAIT);
                ok = 0;
                break;
            }
        }
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

// Sum of nv value-major partials (src[i * nb + t], t < nb) into dst[i], in
// the same order in every CTA: each warp loads 8 values' partials at once
// (one round trip to L2 for up to 32 values per CTA) and sums them with one
// transposed butterfly.
__device__ __forceinline__ void reduce_all(const double *src, int nb, int nv, double *dst) {
    reduce_slots(src, nb, nb, nv, dst);
    __syncthreads();
}

struct CycTile { int prob, rank, nb, row0, row1, pad; };

// One panel of the projection: columns c0 .. c0 + CC (CC <= 8) of V
// against w over the CTA's rows, per-thread sums, then one transposed warp
// reduction into wsum[warp][column].  CC is a compile-time count, so no FP64
// instruction is issued for an absent column (predicated-off FP64
// instructions still occupy GB300's narrow FP64 pipe).  Every present
// column's sum is formed in the same order whatever CC is.
template <int CC>
__device__ __forceinline__ void cyc_proj_panel(const double *__restrict__ V, size_t ld, int c0, int row0, int row1,
                                               const double *__restrict__ w, double (*wsum)[MAXNCV + 1]) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    double a[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) a[q] = 0.0;
    for (int r = row0 + tid; r < row1; r += CTPB) {
        const double wr = w[r];
        const double *vr = V + (size_t)c0 * ld + r;
        double va[CC];
#pragma unroll
        for (int q = 0; q < CC; ++q) va[q] = vr[(size_t)q * ld];
#pragma unroll
        for (int q = 0; q < CC; ++q) a[q] = fma(va[q], wr, a[q]);
    }
    const int q = lane >> 2;
    const double v = warp_reduce8(a);
    if ((lane & 3) == 0 && q < CC) wsum[warp][c0 + q] = v;
}

__device__ __forceinline__ void cyc_proj_panel_n(int cc, const double *__restrict__ V, size_t ld, int c0, int row0,
                                                 int row1, const double *__restrict__ w, double (*wsum)[MAXNCV + 1]) {
    switch (cc) {
    case 1: cyc_proj_panel<1>(V, ld, c0, row0, row1, w, wsum); break;
    case 2: cyc_proj_panel<2>(V, ld, c0, row0, row1, w, wsum); break;
    case 3: cyc_proj_panel<3>(V, ld, c0, row0, row1, w, wsum); break;
    case 4: cyc_proj_panel<4>(V, ld, c0, row0, row1, w, wsum); break;
    case 5: cyc_proj_panel<5>(V, ld, c0, row0, row1, w, wsum); break;
    case 6: cyc_proj_panel<6>(V, ld, c0, row0, row1, w, wsum); break;
    case 7: cyc_proj_panel<7>(V, ld, c0, row0, row1, w, wsum); break;
    default: cyc_proj_panel<8>(V, ld, c0, row0, row1, w, wsum); break;
    }
}

// acc -= V[r, k .. k + R) h[k .. k + R), loads first, in column order.
template <int R>
__device__ __forceinline__ double cyc_update_fp64(const double *__restrict__ vr, size_t ld, int k, const double *hs,
                                                  double acc) {
    double v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = vr[(size_t)(k + q) * ld];
#pragma unroll
    for (int q = 0; q < R; ++q) acc = fma(-v[q], hs[k + q], acc);
    return acc;
}

__device__ __forceinline__ double cyc_update_fp64_n(int cnt, const double *__restrict__ vr, size_t ld, int k,
                                                    const double *hs, double acc) {
    switch (cnt) {
    case 1: return cyc_update_fp64<1>(vr, ld, k, hs, acc);
    case 2: return cyc_update_fp64<2>(vr, ld, k, hs, acc);
    case 3: return cyc_update_fp64<3>(vr, ld, k, hs, acc);
    case 4: return cyc_update_fp64<4>(vr, ld, k, hs, acc);
    case 5: return cyc_update_fp64<5>(vr, ld, k, hs, acc);
    case 6: return cyc_update_fp64<6>(vr, ld, k, hs, acc);
    case 7: return cyc_update_fp64<7>(vr, ld, k, hs, acc);
    default: return cyc_update_fp64<8>(vr, ld, k, hs, acc);
    }
}

template <bool F32>
__device__ __forceinline__ double cyc_spmv_row(const Problem &P, const double *__restrict__ rin, double t1, int r) {
    const int a = P.row_ptr[r], b = P.row_ptr[r + 1];
    if constexpr (F32) {
        float acc = 0.0f;
        for (int i = a; i < b; i += 8) {
            float xv[8], vv[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const bool ok = i + q < b;
                vv[q] = ok ? P.val32[i + q] : 0.0f;
                xv[q] = ok ? (float)(rin[P.col[i + q]] * t1) : 0.0f;
            }
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (i + q < b) acc = fmaf(vv[q], xv[q], acc);
        }
        return (double)acc;
    } else {
        double acc = 0.0;
        for (int i = a; i < b; i += 8) {
            double xv[8], vv[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const bool ok = i + q < b;
                vv[q] = ok ? P.val[i + q] : 0.0;
                xv[q] = ok ? rin[P.col[i + q]] : 0.0;
            }
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (i + q < b) acc = fma(vv[q], xv[q], acc);
        }
        return acc * t1;
    }
}

__global__ void __launch_bounds__(CTPB) k_cycle(const Problem *__restrict__ probs,
                                                const CycTile *__restrict__ tiles, unsigned *__restrict__ bars,
                                                double *__restrict__ xpart, int steps) {
    const CycTile T = tiles[blockIdx.x];
    const Problem &P = probs[T.prob];
    State *S = P.st;
    if (S->status != ST_RUNNING || S->phase != PH_EXTEND || P.wext) return;
    const int k0 = S->k, np = S->np, m = P.ncv;
    const int wl = S->wait_limit;
    const unsigned limit = wl == 0 ? (unsigned)WAIT_LIMIT_DEFAULT : (wl < 0 ? 0u : (unsigned)wl);
    const unsigned nb = (unsigned)T.nb;
    unsigned *bar = bars + T.prob;
    unsigned target = 0;
    const size_t ld = (size_t)P.ld;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row0 = T.row0, row1 = T.row1;
    // partial sums of the group, value-major (i * nb + rank), in three
    // regions of their own: projection, update norm, and the second
    // projection with the first update's norm (CTAs still reading one
    // region after a barrier are never overwritten)
    double *gbase = xpart + (size_t)(blockIdx.x - T.rank) * (3 * (MAXNCV + 2));
    double *partA = gbase;
    double *partB = gbase + (size_t)(MAXNCV + 2) * nb;
    double *partC = gbase + (size_t)(2 * (MAXNCV + 2)) * nb;
    const bool lead = T.rank == 0;

    __shared__ double wsum[CTPB / 32][MAXNCV + 1];
    __shared__ double hs[MAXNCV + 1], red[MAXNCV + 1];
    __shared__ float h32s[MAXNCV];
    __shared__ int s_ok, s_t;

    double rn = S->rnorm;             // norm of the residual the next step normalises
    long long add_passes = 0, add_sumc = 0, add_sumt = 0, add_spmv = 0;
    bool failed = false;
    for (int s = 0; s < steps && s < np; ++s) {
        const int j = k0 + s, c = j + 1;
        const bool scale = rn > DBL_MIN;
        const double t1 = scale ? 1.0 / rn : 1.0;
        const double *__restrict__ rin = step_in(P, j);
        double *__restrict__ w = step_out(P, j);
        // ---- SpMV of own rows (HLanc.hpp:1424) ----------------------------------
        for (int r = row0 + tid; r < row1; r += CTPB) {
            const double x = rin[r];
            const double v = scale ? x * t1 : x;
            const double y = P.fp32 ? cyc_spmv_row<true>(P, rin, t1, r) : cyc_spmv_row<false>(P, rin, t1, r);
            w[r] = y;
            P.V[(size_t)j * ld + r] = v;
            P.V32[(size_t)j * ld + r] = (float)v;
        }
        ++add_spmv;
        double wnorm = 0.0;
        // Projection partials of own rows, h = V[:, 0:c)^T w (+ ||w||^2 with
        // `norm` at index c), summed over the CTA and written to dst[i * nb + rank].
        auto proj_partials = [&](bool norm, double *dst) {
            __syncthreads();   // w of own rows complete (written by other threads)
            double nrm = 0.0;
            if (norm)
                for (int r = row0 + tid; r < row1; r += CTPB) nrm = fma(w[r], w[r], nrm);
            int c0 = 0;
            for (; c0 + 16 <= c; c0 += 16) {          // full rounds: two panels of 8
                double a[8], b[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) a[q] = b[q] = 0.0;
                for (int r = row0 + tid; r < row1; r += CTPB) {
                    const double wr = w[r];
                    const double *vr = P.V + (size_t)c0 * ld + r;
                    double va[8], vb[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        va[q] = vr[(size_t)q * ld];
                        vb[q] = vr[(size_t)(q + 8) * ld];
                    }
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        a[q] = fma(va[q], wr, a[q]);
                        b[q] = fma(vb[q], wr, b[q]);
                    }
                }
                const double v = warp_reduce8(a);
                const double u = warp_reduce8(b);
                const int q = lane >> 2;
                if ((lane & 3) == 0) {
                    wsum[warp][c0 + q] = v;
                    wsum[warp][c0 + 8 + q] = u;
                }
            }
            for (; c0 < c; c0 += 8)                     // the rest, panels of exactly the remaining columns
                cyc_proj_panel_n(min(8, c - c0), P.V, ld, c0, row0, row1, w, wsum);
            if (norm) {
                nrm = warp_sum(nrm);
                if (lane == 0) wsum[warp][c] = nrm;
            }
            __syncthreads();
            const int nv = c + (norm ? 1 : 0);
            for (int i = tid; i < nv; i += CTPB) {
                double t = 0.0;
#pragma unroll
                for (int q = 0; q < CTPB / 32; ++q) t += wsum[q][i];
                dst[(size_t)i * nb + T.rank] = t;
            }
        };
        // The second pass's projection is computed together with the norm
        // of the first update (one barrier for both): nearly every step
        // needs a second pass, and both read only own rows.  red holds it
        // when `pre` is set.
        bool pre = false;
        for (int pass = 1; pass <= 3; ++pass) {
            if (!pre) {
                proj_partials(pass == 1, partA);
                if (!group_sync(bar, nb, target, limit, S, &s_ok)) { failed = true; break; }
                reduce_all(partA, (int)nb, c + (pass == 1 ? 1 : 0), red);
            }
            pre = false;
            double *h = P.small + SM_H(m);
            if (pass == 1) {
                wnorm = sqrt(red[c]);                             // HLanc.hpp:1429
                if (lead && tid == 0) {
                    h[m + j] = red[j];                            // alpha_j, HLanc.hpp:1433
                    h[j] = (j == 0) ? 0.0 : rn;                   // beta_j,  HLanc.hpp:1434-1438
                }
            } else if (lead && tid == 0) {
                h[m + j] += red[j];                               // HLanc.hpp:1447
            }
            ++add_passes;
            // ---- update w -= V h of own rows (FP32 copy for small coefficients) ----
            const double sc = pass == 1 ? wnorm : rn;
            const bool usable = sc > 0.0 && sc <= DBL_MAX;
            const double thr = usable ? ldexp(sc, -32) / c : 0.0;
            if (tid == 0) s_t = usable ? c : 0;
            __syncthreads();
            for (int i = tid; i < c; i += CTPB) {
                hs[i] = red[i];
                if (usable && !(fabs(red[i]) <= thr)) atomicMin(&s_t, i);
            }
            __syncthreads();
            const int tf = s_t;
            const int ke = usable ? -ilogb(sc) : 0;
            for (int i = tid; i < tf; i += CTPB) h32s[i] = (float)ldexp(hs[i], ke);
            __syncthreads();
            const double unscale = ldexp(1.0, -ke);
            double nrm2 = 0.0;
            for (int r = row0 + tid; r < row1; r += CTPB) {
                double acc = w[r];
                // columns 8 at a time, loads issued before the FMAs
                float a32 = 0.0f;
                for (int i0 = 0; i0 < tf; i0 += 8) {
                    float v[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) v[q] = i0 + q < tf ? P.V32[(size_t)(i0 + q) * ld + r] : 0.0f;
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        if (i0 + q < tf) a32 = fmaf(v[q], h32s[i0 + q], a32);
                }
                acc = fma(-(double)a32, unscale, acc);
                for (int i0 = tf; i0 < c; i0 += 8)
                    acc = cyc_update_fp64_n(min(8, c - i0), P.V + r, ld, i0, hs, acc);
                w[r] = acc;
                nrm2 = fma(acc, acc, nrm2);
            }
            add_sumc += c;
            add_sumt += tf;
            const bool fuse = pass == 1;
            if (fuse) {
                proj_partials(true, partC);
            } else {
                nrm2 = warp_sum(nrm2);
                __syncthreads();
                if (lane == 0) wsum[warp][0] = nrm2;
                __syncthreads();
                if (tid == 0) {
                    double t = 0.0;
#pragma unroll
                    for (int q = 0; q < CTPB / 32; ++q) t += wsum[q][0];
                    partB[T.rank] = t;
                }
            }
            if (!group_sync(bar, nb, target, limit, S, &s_ok)) { failed = true; break; }
            if (fuse) reduce_all(partC, (int)nb, c + 1, red);
            else reduce_all(partB, (int)nb, 1, red);
            const double nr = sqrt(red[fuse ? c : 0]);
            // ---- DGKS decision (HLanc.hpp:1440-1463), identical in every CTA ----
            bool again;
            if (pass == 1) {
                rn = nr;
                again = nr < wnorm * 0.717;
            } else if (pass == 2) {
                again = !(nr > rn * 0.717);
                rn = nr;
            } else {
                again = false;
                if (nr > rn * 0.717) {
                    rn = nr;
                } else {                                          // invariant subspace: resid = 0
                    rn = 0.0;
                    for (int r = row0 + tid; r < row1; r += CTPB) w[r] = 0.0;
                    if (!group_sync(bar, nb, target, limit, S, &s_ok)) { failed = true; break; }
                }
            }
            if (lead && tid == 0) {
                S->rnorm = rn;
                if (pass == 1) { S->wnorm = wnorm; S->need2 = again; S->need3 = 0; }
                else if (pass == 2) S->need3 = again;
            }
            if (!again) break;
            pre = fuse;
        }
        if (failed) break;
    }
    if (lead && tid == 0) {
        S->spmv += add_spmv;
        S->passes += add_passes;
        S->sumc += add_sumc;
        S->sumt += add_sumt;
    }
}

// ---- launcher --------------------------------------------------------------
// Largest grid of k_cycle that is co-resident on this device (0 if the
// device cannot run cooperative launches).
int cycle_capacity() {
    int dev = 0, coop = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_cycle, CTPB, 0) != cudaSuccess) return 0;
    cudaGetLastError();
    return per * sms;
}

// Rows per CTA of a problem's group.  Measured on the 10,000-row 2-D
// Laplacian (whole solves): 128 rows 192 eigenpairs/s, 256 rows 167, 64
// rows 182, 32 rows 129 -- fewer rows per CTA add barrier arrivals and
// partials to reduce faster than they remove work per CTA.
int cycle_rows_per_cta() { return CTPB; }

cudaError_t launch_cycle(const Problem *P_d, const void *tiles_d, int nctas, unsigned *bars_d, double *xpart_d,
                         int nprob, int steps, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(bars_d, 0, sizeof(unsigned) * (size_t)nprob, s);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nctas);
    cfg.blockDim = dim3(CTPB);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    prof_begin(s);
    e = cudaLaunchKernelEx(&cfg, k_cycle, P_d, static_cast<const CycTile *>(tiles_d), bars_d, xpart_d, steps);
    prof_end(KC_CYCLE, s);
    launch_counter() += 1;
    variant_counter(HLANC_KL_CYCLE) += 1;
    return e;
}

}  // namespace hlanc
