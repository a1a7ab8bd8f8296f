// kernels_tc.cu -- the restart's basis update V[:, 0:nev) <- V Q on the
// fifth-generation tensor cores (tcgen05), accurate to FP64 level.
//
// GB300 runs FP64 FMAs at 2 per clock per SM on the CUDA cores, so the
// FP64 form of this update (k_basis: ~nev + np FMAs per output) is
// FP64-bound.  Here the product is computed exactly in integer arithmetic
// on the f16 tensor pipe (the splitting idea of Ozaki et al., "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication", Numer. Algorithms 2012):
//
//  * every row r of the 128-row block of V gets the exponent E_r of its
//    largest element; each element becomes the integer |X| = |v| 2^(55-E_r)
//    (truncated, < 2^55) with the element's sign, i.e. 7 unsigned 8-bit
//    digits a_0 (most significant) .. a_6, each stored as a signed f16
//    (exact: |digit| <= 255 needs 8 significand bits);
//  * every output column i of Q (the band of Q[:, i], i < nev, and the
//    residual column Q[:, nev]) is split the same way with its own exponent;
//  * D_L = sum over s + t = L of A_s B_t (L = 0..6) accumulates in FP32 in
//    tensor memory.  Digit products are < 2^16 and K <= 64, so a pair sum is
//    < 2^22 and levels 0..3 (at most 4 pairs) stay below 2^24: exact.  The
//    lower levels can round by a few units at weights 2^-32 .. 2^-48 of
//    level 0, i.e. below FP64 precision.  Levels past 6 are dropped
//    (weight <= 2^-56 of the result's scale).
//  * the levels are recombined per output in 64-bit integers, placed
//    exactly into two doubles through their bit patterns, and added: two
//    FP64 instructions per output instead of ~50 FMAs.
//  * plane s of V only feeds levels s..6, so each plane's MMA covers N =
//    (7 - s) * NPAD accumulator columns.
//
// Shapes: M = 128 rows per MMA, NPAD = nev + 1 padded to 16 (<= 64), K =
// ncv padded to 16 (<= 64).  Operands live in shared memory in the
// no-swizzle K-major layout (8-row x 16-byte core matrices); the
// accumulators (7 x NPAD columns) in tensor memory.  One CTA per tile of
// rows, one CTA per SM.  Measured on GB300 at n = 4.1M, ncv = 60: 2.7 ms
// (nev 20) and 3.8 ms (nev 40) against 8.8 / 17.8 ms for the FP64 kernel.
// k_basis_tc2 (below) runs the same products with the phases of
// consecutive blocks overlapped by warp role, for nev + 1 <= 32 (2.3 ms at
// nev 20, same shape).
//
// The same splitting was tried for the CGS passes (w -= V h, h = V^T w),
// where each element of V meets a single output: the splitting alone costs
// more issue slots per element than the FP64 kernels' DFMA, so those stay
// on the FP64 pipe.
#include <cuda_fp16.h>

#include "internal.cuh"

namespace hlanc {

namespace tc {

constexpr int BM = 128;       // rows per block = MMA M
constexpr int NDIG = 7;       // digit planes / levels
constexpr int KMAX = 64;      // largest padded ncv
constexpr int NMAX = 64;      // largest padded nev + 1
constexpr int THREADS = 512;
constexpr int NQ = THREADS / BM;   // threads per row of a block (each loads and splits 1/NQ of its columns)
constexpr int GMAX = (KMAX / 8 + NQ - 1) / NQ;   // 8-column groups per thread

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor, no swizzle: start, leading byte offset
// (next core matrix along K), stride byte offset (next 8 rows), version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: D f32, A/B f16, both K-major.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                    uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(mbar))
                 : "memory");
}
__device__ __forceinline__ void mbar_init(uint64_t *m, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *m, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(m)), "r"(parity)
        : "memory");
    return ok != 0;
}
// The same test, with the thread suspended until the phase completes or
// about `ns` nanoseconds pass (a waiting warp then issues nothing, instead
// of spinning on the test and taking issue slots from the working warps).
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t *m, uint32_t parity, uint32_t ns) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(m)), "r"(parity), "r"(ns)
        : "memory");
    return ok != 0;
}
// Levels 0..6 of 4 consecutive outputs of this thread's TMEM lane: seven
// 32x32b.x4 loads (level L at column offset L * npad) and one wait, in one
// asm block so the registers are read only after the wait.
__device__ __forceinline__ void tmem_ld_levels4(uint32_t a, uint32_t npad, float (&d)[NDIG][4]) {
    uint32_t r[NDIG * 4];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%28];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%4,%5,%6,%7}, [%29];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%8,%9,%10,%11}, [%30];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%12,%13,%14,%15}, [%31];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%16,%17,%18,%19}, [%32];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%20,%21,%22,%23}, [%33];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%24,%25,%26,%27}, [%34];\n\t"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27])
        : "r"(a), "r"(a + npad), "r"(a + 2 * npad), "r"(a + 3 * npad), "r"(a + 4 * npad), "r"(a + 5 * npad),
          "r"(a + 6 * npad)
        : "memory");
#pragma unroll
    for (int L = 0; L < NDIG; ++L)
#pragma unroll
        for (int e = 0; e < 4; ++e) d[L][e] = __uint_as_float(r[L * 4 + e]);
}

// Start streaming rows [r0, r0 + rows) of the first m columns of V into L2
// (one bulk prefetch per column, issued by threads 0..m-1).  V's columns
// are 512-byte aligned and at least an even number of rows long past any
// tile row, so rows is rounded up to an even count (16-byte multiple).
__device__ __forceinline__ void prefetch_rows_l2(const double *V, size_t ld, int m, int r0, int rows) {
    const int k = threadIdx.x;
    if (rows <= 0 || k >= m) return;
    const unsigned bytes = (unsigned)(((rows + 1) & ~1) * 8);
    const double *p = V + r0 + (size_t)k * ld;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Byte offset of element (row, k) in a no-swizzle K-major operand with
// kpad columns: core matrix (row/8, k/8) at (row/8)*SBO + (k/8)*128,
// SBO = (kpad/8)*128; inside, row%8 at 16 B, k%8 at 2 B.
__device__ __forceinline__ uint32_t kmajor_off(int row, int k, int kpad) {
    return (uint32_t)((row >> 3) * (kpad >> 3) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// Biased exponent field of a double (0 for zero and subnormals).
__device__ __forceinline__ int exp_field(double x) {
    return (int)((__double_as_longlong(x) >> 52) & 0x7FF);
}

// |X| = (mantissa << 2) >> (emax - e) < 2^55 of one element, relative to the
// largest biased exponent emax of its row / column, as two words, and its
// sign.  32-bit funnel shifts on the two halves of the mantissa (a 64-bit
// variable shift costs several instructions more per element).
__device__ __forceinline__ void split_mag(double x, int emax, unsigned &lo, unsigned &hi, bool &neg) {
    const unsigned bh = (unsigned)__double2hiint(x), bl = (unsigned)__double2loint(x);
    const int ex = (int)((bh >> 20) & 0x7FFu);
    neg = (bh >> 31) != 0u;
    const unsigned mh = (((bh & 0xFFFFFu) | 0x100000u) << 2) | (bl >> 30);   // bits 32..54 of mantissa << 2
    const unsigned ml = bl << 2;
    const int sh = emax - ex;
    lo = 0u;
    hi = 0u;
    if (ex != 0) {
        if (sh < 32) {
            lo = __funnelshift_r(ml, mh, (unsigned)sh);
            hi = mh >> sh;
        } else if (sh < 64) {
            lo = mh >> (sh - 32);
        }
    }
}

// Digit plane q (0 = most significant) of 8 elements -- byte 6 - q of each
// |X| with the element's sign -- as 4 words of f16 pairs.  A byte d becomes
// the f16 1024 + d by placing it under the exponent of 1024 (0x64 in the
// high byte of each half), and one f16x2 FMA per pair, (1024 + d) s -
// 1024 s, gives s d exactly (|d| <= 255 is exact in f16): a permute, a
// logic operation and an FMA per two digits, no conversion instruction (on
// GB300 conversions share the narrow FP64 pipe).
struct Signs8 {
    unsigned sg[4], ns[4];   // per pair: (+-1, +-1) and (-+1024, -+1024) as f16x2
};
__device__ __forceinline__ void signs8(const bool (&ng)[8], Signs8 &S) {
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        S.sg[p] = (ng[2 * p] ? 0xBC00u : 0x3C00u) | ((ng[2 * p + 1] ? 0xBC00u : 0x3C00u) << 16);
        S.ns[p] = (ng[2 * p] ? 0x6400u : 0xE400u) | ((ng[2 * p + 1] ? 0x6400u : 0xE400u) << 16);
    }
}
__device__ __forceinline__ uint4 plane8(const unsigned (&lo)[8], const unsigned (&hi)[8], const Signs8 &S, int q) {
    const unsigned b = (unsigned)(q < 3 ? 2 - q : 6 - q);
    const unsigned sel = b | ((b + 4u) << 8);     // byte b of the pair's first word -> byte 0, second -> byte 2
    unsigned w[4];
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        const unsigned a0 = q < 3 ? hi[2 * p] : lo[2 * p], a1 = q < 3 ? hi[2 * p + 1] : lo[2 * p + 1];
        const unsigned t = (__byte_perm(a0, a1, sel) & 0x00FF00FFu) | 0x64006400u;
        unsigned r;
        asm("fma.rn.f16x2 %0, %1, %2, %3;" : "=r"(r) : "r"(t), "r"(S.sg[p]), "r"(S.ns[p]));
        w[p] = r;
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// The 7 digits of 8 elements as f16 pairs: 7 x uint4.
__device__ __forceinline__ void split8(const double (&x)[8], int emax, uint4 (&planes)[NDIG]) {
    unsigned lo[8], hi[8];
    bool ng[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) split_mag(x[e], emax, lo[e], hi[e], ng[e]);
    Signs8 S;
    signs8(ng, S);
#pragma unroll
    for (int q = 0; q < NDIG; ++q) planes[q] = plane8(lo, hi, S, q);
}

// The integer value of an integer-valued FP32 level (|x| < 2^25: at most 7
// digit-pair sums of 64 products below 2^16) from its bit pattern, with
// 32-bit integer instructions only (a level sum of integer products is an
// integer: below 2^24 it is exact, above it every FP32 value is an integer).
__device__ __forceinline__ long long level_int(float f) {
    const unsigned u = __float_as_uint(f);
    const int e = (int)((u >> 23) & 0xFFu);
    if (e < 127) return 0;                         // |f| < 1: zero
    const int m = (int)((u & 0x7FFFFFu) | 0x800000u);
    const int sh = e - 150;                        // |f| = m 2^sh, sh <= 1
    const int v = sh >= 0 ? (m << sh) : (m >> (-sh));
    return (long long)((u >> 31) ? -v : v);
}

// Levels D_0..D_6 (exact integers in FP32) of one output -> the FP64 value
// (hi 2^32 + lo) 2^S with hi = D_0 2^16 + D_1 2^8 + D_2, lo = D_3 2^24 +
// D_4 2^16 + D_5 2^8 + D_6 and S = ex + fx - 2106 (ex, fx: the biased
// exponents the row and the column were split against).  Both halves are
// placed exactly into doubles by adding them to the significand of
// A0 = 1.5 * 2^(84+S) resp. B0 = 1.5 * 2^(52+S) (|hi|, |lo| < 2^51).
// A0 + B0 fits in 35 significant bits, so (A - (A0 + B0)) is exact and
// the value costs two FP64 additions with one rounding.
__device__ __forceinline__ double combine(const float (&d)[NDIG], int ex, int fx) {
    // every level is an integer below 2^25 in magnitude
    const long long l0 = level_int(d[0]), l1 = level_int(d[1]), l2 = level_int(d[2]);
    const long long l3 = level_int(d[3]), l4 = level_int(d[4]), l5 = level_int(d[5]);
    const long long l6 = level_int(d[6]);
    const long long hi = (l0 << 16) + (l1 << 8) + l2;                 // |hi| < 2^41
    const long long lo = (l3 << 24) + (l4 << 16) + (l5 << 8) + l6;    // |lo| < 2^50
    const int S = ex + fx - 2106;
    const long long eA = 1023 + 84 + S, eB = 1023 + 52 + S;           // biased exponents of the carriers
    if (eB >= 1 && eA <= 2046) {
        const long long half = 1LL << 51;                             // 1.5 = 1 + 2^-1
        const double A = __longlong_as_double((eA << 52) + half + hi);
        const double B = __longlong_as_double((eB << 52) + half + lo);
        // A0 + B0: B0 is 1.5 * 2^20 units of A0's last place (2^(32+S))
        const double cAB = __longlong_as_double((eA << 52) + half + (3LL << 19));
        return (A - cAB) + B;
    }
    return scalbn(fma((double)hi, 4294967296.0, (double)lo), S);
}

}  // namespace tc

// One CTA per tile; 128-row blocks of the tile in turn.
// RITZ: the same product for the Ritz vectors of a converged problem,
// vout[:, 0:ncv) = V Q2 with the dense ncv x ncv factor Q2
// (HLanc.hpp:1840-1843): every column of Q2 is an output, there is no
// residual column, and nothing of the basis is overwritten.
template <int NPAD, bool RITZ>
__global__ void __launch_bounds__(tc::THREADS, 1) k_basis_tc(const Problem *__restrict__ probs,
                                                            const Tile *__restrict__ tiles) {
    using namespace tc;
    const Tile t = tiles[blockIdx.x];
    const Problem &P = probs[t.prob];
    State *S = P.st;
    if (RITZ ? (S->status != ST_CONVERGED || S->fin != 1) : (S->status != ST_RUNNING || S->phase != PH_APPLY))
        return;
    const int m = P.ncv, nev = S->nev, np = S->np;
    const int wl = S->wait_limit;
    const unsigned wait_limit = wl == 0 ? (unsigned)WAIT_LIMIT_DEFAULT : (wl < 0 ? 0u : (unsigned)wl);
    const int kpad = (m + 15) & ~15;
    const int nout = RITZ ? m : nev + 1;
    constexpr uint32_t NCOLS = (NDIG * NPAD > 256) ? 512u : (NDIG * NPAD > 128 ? 256u : 128u);

    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sA = smem;                                   // NDIG x BM x kpad f16
    // Q's digit planes stacked: rows t * NPAD + i hold plane t of output i
    // (t = 0..6).  Plane s of V contributes to levels L = s..6 only, so its
    // MMA writes accumulator columns [s * NPAD, 7 * NPAD) with the stack's
    // first (7 - s) * NPAD rows as B: column block L meets plane L - s.
    unsigned char *sB = smem + (size_t)NDIG * BM * KMAX * 2;    // 7 x NPAD x kpad f16
    __shared__ uint64_t s_mbar;
    __shared__ uint32_t s_taddr;
    __shared__ int s_rowexp[NQ][BM];
    __shared__ int s_colexp[NPAD];
    __shared__ double s_red[32], s_mine[1], s_tot[1];
    __shared__ int s_fail;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const double *Q = P.small + (RITZ ? SM_Q2(m) : SM_Q(m));
    const double *h = P.small + SM_H(m);
    const size_t aplane = (size_t)BM * kpad * 2, bplane = (size_t)NPAD * kpad * 2;

    prefetch_rows_l2(P.V, (size_t)P.ld, m, t.row0, min(BM, t.row1 - t.row0));
    if (warp == 0) {
        tmem_alloc(&s_taddr, NCOLS);
        tmem_relinquish();
    }
    if (tid == 0) {
        mbar_init(&s_mbar, 1);
        s_fail = 0;
    }
    for (int i = tid; i < NPAD; i += THREADS) s_colexp[i] = 0;
    __syncthreads();

    // ---- B planes: the output columns of Q, split per column -------------------
    // column i < nev: Q[k, i] for k <= i + np (the band), i == nev: Q[:, nev];
    // RITZ: every column of Q2, dense
    auto qval = [&](int k, int i) -> double {
        if (i >= nout || k >= m) return 0.0;
        if (!RITZ && i < nev && k > i + np) return 0.0;
        return Q[k + (size_t)i * m];
    };
    const int kg = kpad >> 3;
    for (int it = tid; it < NPAD * kg; it += THREADS) {
        const int i = it / kg, g = it % kg;
        int emax = 0;
        for (int e = 0; e < 8; ++e) emax = max(emax, exp_field(qval(8 * g + e, i)));
        atomicMax(&s_colexp[i], emax);
    }
    __syncthreads();
    for (int it = tid; it < NPAD * kg; it += THREADS) {
        const int i = it / kg, g = it % kg;
        double x[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) x[e] = qval(8 * g + e, i);
        uint4 pl[NDIG];
        split8(x, s_colexp[i], pl);
        const uint32_t off = kmajor_off(i, 8 * g, kpad);
#pragma unroll
        for (int s = 0; s < NDIG; ++s) *reinterpret_cast<uint4 *>(sB + s * bplane + off) = pl[s];
    }


    const uint32_t sbo = (uint32_t)kg * 128u;
    const uint32_t taddr = s_taddr;
    const double hn = RITZ ? 0.0 : h[nev];
    const double qlast = RITZ ? 0.0 : Q[(m - 1) + (size_t)(nev - 1) * m];
    const double *__restrict__ rin = (m & 1) ? P.r1 : P.r0;
    double *__restrict__ rout = (nev & 1) ? P.r1 : P.r0;
    const size_t ld = (size_t)P.ld, ldo = (size_t)P.ldo;
    double nrm = 0.0;
    uint32_t phase = 0;

    // loader mapping: row r of the block, groups g0.. of 8 columns
    const int lr = tid & (BM - 1), part = tid / BM;
    const int gper = (kg + NQ - 1) / NQ, g0 = part * gper, g1 = min(kg, g0 + gper);

    // this thread's part of row R0 + lr (zeros past the tile / past ncv)
    auto load_rows = [&](int R0, double (&x)[GMAX][8]) {
        const int row = R0 + lr;
        const bool rok = row < t.row1;
#pragma unroll
        for (int q = 0; q < GMAX; ++q) {
            const int g = g0 + q;
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int k = 8 * g + e;
                x[q][e] = (rok && g < g1 && k < m) ? P.V[row + (size_t)k * ld] : 0.0;
            }
        }
    };
    double x[GMAX][8];
    prefetch_rows_l2(P.V, ld, m, t.row0 + BM, min(BM, t.row1 - (t.row0 + BM)));
    load_rows(t.row0, x);

    for (int R0 = t.row0; R0 < t.row1; R0 += BM) {
        prefetch_rows_l2(P.V, ld, m, R0 + 2 * BM, min(BM, t.row1 - (R0 + 2 * BM)));
        // 1. the largest exponent of each row (x holds this block, loaded
        //    while the previous block's products ran)
        int emax = 0;
#pragma unroll
        for (int q = 0; q < GMAX; ++q)
#pragma unroll
            for (int e = 0; e < 8; ++e) emax = max(emax, exp_field(x[q][e]));
        s_rowexp[part][lr] = emax;
        __syncthreads();
        int ex = s_rowexp[0][lr];
#pragma unroll
        for (int q = 1; q < NQ; ++q) ex = max(ex, s_rowexp[q][lr]);
        // 2. digit planes of the block
#pragma unroll
        for (int q = 0; q < GMAX; ++q) {
            const int g = g0 + q;
            if (g >= g1) break;
            uint4 pl[NDIG];
            split8(x[q], ex, pl);
            const uint32_t off = kmajor_off(lr, 8 * g, kpad);
#pragma unroll
            for (int s = 0; s < NDIG; ++s) *reinterpret_cast<uint4 *>(sA + s * aplane + off) = pl[s];
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        // 3. one thread issues the 28 digit-pair products per K step
        if (tid == 0) {
            fence_after();
            const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
            for (int s = 0; s < NDIG; ++s) {
                // N = (7 - s) * NPAD columns, in one MMA or two (each <= 256, a multiple of 16)
                const int ns = (NDIG - s) * NPAD;
                const int n1 = ns <= 256 ? ns : ((ns / 2 + 15) / 16) * 16, n2 = ns - n1;
                const uint32_t id1 = instr_desc(BM, n1), id2 = instr_desc(BM, n2 > 0 ? n2 : 16);
                const uint32_t d0 = taddr + (uint32_t)(s * NPAD);
                const uint32_t n1_bytes = (uint32_t)(n1 / 8) * sbo;   // n1 rows further in the stack
                for (int kk = 0; kk < kpad / 16; ++kk) {
                    const uint64_t ad = smem_desc(a0 + (uint32_t)(s * aplane) + kk * 256u, 128u, sbo);
                    const uint32_t acc = (s | kk) ? 1u : 0u;
                    mma(d0, ad, smem_desc(b0 + kk * 256u, 128u, sbo), id1, acc);
                    if (n2 > 0) mma(d0 + (uint32_t)n1, ad, smem_desc(b0 + n1_bytes + kk * 256u, 128u, sbo), id2, acc);
                }
            }
            mma_commit(&s_mbar);
        }
        // 3b. the next block's rows load while the products run (x is free
        //     after the split; the recombine below writes other rows)
        if (R0 + BM < t.row1) load_rows(R0 + BM, x);
        // 4. wait for the products (bounded).  A wait that gives up marks the
        //    CTA failed, then waits (again bounded) for the MMAs it already
        //    issued, so tensor memory is not released under them.
        {
            bool done = false;
            for (unsigned spins = 0; spins < wait_limit; ++spins)
                if (mbar_try_wait_sleep(&s_mbar, phase, 1000u)) { done = true; break; }
            if (!done) {
                s_fail = 1;
                for (unsigned spins = 0; spins < (unsigned)WAIT_LIMIT_DEFAULT; ++spins)
                    if (mbar_try_wait(&s_mbar, phase)) break;
            }
        }
        phase ^= 1u;
        fence_after();
        __syncthreads();
        if (s_fail) break;
        // 5. recombine: warp w reads TMEM lanes 32 (w % 4) .. +31; the four warps of a
        //    lane quarter take every fourth group of 4 outputs
        {
            const int q4 = warp & 3, ch = warp >> 2;
            const int r = 32 * q4 + lane;
            const int orow = R0 + r;
            const bool ok = orow < t.row1;
            int exr = s_rowexp[0][r];
#pragma unroll
            for (int q = 1; q < NQ; ++q) exr = max(exr, s_rowexp[q][r]);
            const uint32_t lane_base = taddr + ((uint32_t)(32 * q4) << 16);
            for (int c0 = ch * 4; c0 < nout; c0 += 4 * (THREADS / 128)) {
                float d[NDIG][4];
                tmem_ld_levels4(lane_base + (uint32_t)c0, (uint32_t)NPAD, d);
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int i = c0 + e;
                    if (i >= nout || !ok) continue;
                    float lv[NDIG];
#pragma unroll
                    for (int L = 0; L < NDIG; ++L) lv[L] = d[L][e];
                    const double v = combine(lv, exr, s_colexp[i]);
                    if (RITZ) {
                        P.vout[orow + (size_t)i * ldo] = v;
                    } else if (i < nev) {
                        P.V[orow + (size_t)i * ld] = v;
                        P.V32[orow + (size_t)i * ld] = (float)v;
                    } else {                                      // residual (HLanc.hpp:1605-1614)
                        double res = rin[orow] * qlast;
                        if (hn > 0.0) res = res + hn * v;
                        rout[orow] = res;
                        nrm = fma(res, res, nrm);
                    }
                }
            }
        }
        fence_before();
        __syncthreads();
    }

    // release tensor memory (all TMEM reads are complete)
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        tmem_dealloc(taddr, NCOLS);
    }
    // A failed CTA still takes part in the tile reduction below, so the tile
    // group's counters are reset for the next launch; the host reads S->err
    // after the cycle and abandons the solve.
    if (s_fail && tid == 0) atomicExch(&S->err, DEV_ERR_MMA_WAIT);
    nrm = block_sum0(nrm, s_red);
    if (tid == 0) s_mine[0] = nrm;
    __syncthreads();
    if (!finish_tile(P, blockIdx.x - P.tile0, 1, s_mine, s_tot)) return;
    if (tid == 0) {
        if (RITZ) {
            S->fin = 2;
        } else {
            S->rnorm = sqrt(s_tot[0]);                // HLanc.hpp:1735
            S->phase = PH_EXTEND;
            S->sumnev += nev;
            S->napply += 1;
        }
    }
}

// ---- warp-specialised form (nev + 1 <= 32) ---------------------------------
// The same products with the phases of consecutive 128-row blocks
// overlapped, instead of run one after another by every thread:
//   warp 16, one thread: bulk copies (cp.async.bulk, one per column) of a
//       block of V into a raw FP64 stage, and the MMAs;
//   warps 0-7, splitters, two threads per row: the row's exponent, then the
//       digit planes of each K half (columns 0-31, 32-63) into that half's
//       A buffer as soon as the previous block's MMAs of the half have read
//       it; the stage is released after the first half, so the next block's
//       copy runs while the second half is split;
//   warps 8-15, recombiners: levels from one of two TMEM accumulators while
//       the next block's MMAs fill the other, recombination and stores.
// mbarriers carry the hand-offs.  Every wait is bounded: one that gives up
// raises s_fail, which the other roles' waits also watch, so every thread
// reaches the end, where the MMAs and bulk copies in flight are drained
// before TMEM and shared memory are released.
namespace tc2 {
constexpr int THREADS = 17 * 32;
constexpr int SPLIT_WARPS = 8, REC_WARPS = 8, CTRL_WARP = 16;
constexpr int KH = 32;                                      // columns per K half
constexpr size_t APLANE = (size_t)tc::BM * KH * 2;          // one digit plane of one half
constexpr size_t ABUF = (size_t)tc::NDIG * APLANE;          // one half's planes (56 KB)
constexpr size_t STAGE = (size_t)tc::BM * tc::KMAX * 8;     // raw FP64 rows of one block (64 KB)
}  // namespace tc2

template <int NPAD>
static size_t basis_tc2_smem() {
    return 2 * tc2::ABUF + (size_t)tc::NDIG * NPAD * tc::KMAX * 2 + tc2::STAGE;
}

namespace tc {
__device__ __forceinline__ void mbar_arrive(uint64_t *m) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(m)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *m, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes)
                 : "memory");
}
// One bulk copy global -> shared (16-byte aligned addresses, size a
// multiple of 16) completing bytes on mbarrier m.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *m) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(m))
                 : "memory");
}
// Bounded wait for the phase of parity `parity`: false after `limit` polls
// (raising *fail) or as soon as another role raised *fail.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *m, uint32_t parity, unsigned limit, volatile int *fail) {
    for (unsigned spins = 0; spins < limit; ++spins) {
        if (mbar_try_wait_sleep(m, parity, 1000u)) return true;
        if (*fail) return false;
    }
    *fail = 1;
    return false;
}
// The 7 digit planes of 8 elements, stored plane by plane (few live registers).
__device__ __forceinline__ void split8_store(const double (&x)[8], int emax, unsigned char *base, uint32_t off) {
    unsigned lo[8], hi[8];
    bool ng[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) split_mag(x[e], emax, lo[e], hi[e], ng[e]);
    Signs8 S;
    signs8(ng, S);
#pragma unroll
    for (int q = 0; q < NDIG; ++q) *reinterpret_cast<uint4 *>(base + q * tc2::APLANE + off) = plane8(lo, hi, S, q);
}
}  // namespace tc

template <int NPAD>
__global__ void __launch_bounds__(tc2::THREADS, 1) k_basis_tc2(const Problem *__restrict__ probs,
                                                              const Tile *__restrict__ tiles) {
    using namespace tc;
    const Tile t = tiles[blockIdx.x];
    const Problem &P = probs[t.prob];
    State *S = P.st;
    if (S->status != ST_RUNNING || S->phase != PH_APPLY) return;
    const int m = P.ncv, nev = S->nev, np = S->np;
    const int wl = S->wait_limit;
    const unsigned limit = wl == 0 ? (unsigned)WAIT_LIMIT_DEFAULT : (wl < 0 ? 0u : (unsigned)wl);
    const int kpad = (m + 15) & ~15;
    const int ksteps = kpad / 16;                           // K = 16 per MMA
    const bool two = ksteps > 2;                            // ncv > 32: the second K half exists
    const int nout = nev + 1;
    constexpr uint32_t ACC = (uint32_t)(NDIG * NPAD);       // columns of one accumulator
    constexpr uint32_t NCOLS = 2 * ACC > 256 ? 512u : 256u;
    const size_t ld = (size_t)P.ld;
    const int nblk = (t.row1 - t.row0 + BM - 1) / BM;

    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sA = smem;                                               // 2 halves x 7 planes
    unsigned char *sB = smem + 2 * tc2::ABUF;                               // 7 x NPAD x kpad
    double *stage = reinterpret_cast<double *>(sB + (size_t)NDIG * NPAD * KMAX * 2);   // [column][128 rows]
    __shared__ uint64_t bar_full, bar_empty, bar_afull[2], bar_aempty[2], bar_accfull[2], bar_accempty[2];
    __shared__ uint64_t bar_drain;
    __shared__ uint32_t s_taddr;
    __shared__ int s_rowexp[4][BM];
    __shared__ int s_colexp[NPAD];
    __shared__ double s_red[32], s_mine[1], s_tot[1];
    __shared__ int s_fail;
    volatile int *fail = &s_fail;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const double *Q = P.small + SM_Q(m);
    const double *h = P.small + SM_H(m);

    if (warp == tc2::CTRL_WARP) {
        tmem_alloc(&s_taddr, NCOLS);
        tmem_relinquish();
    }
    if (tid == 0) {
        s_fail = 0;
        mbar_init(&bar_full, 1);
        mbar_init(&bar_empty, tc2::SPLIT_WARPS);
        mbar_init(&bar_drain, 1);
        for (int q = 0; q < 2; ++q) {
            mbar_init(&bar_afull[q], tc2::SPLIT_WARPS);
            mbar_init(&bar_aempty[q], 1);
            mbar_init(&bar_accfull[q], 1);
            mbar_init(&bar_accempty[q], tc2::REC_WARPS);
        }
    }
    for (int i = tid; i < NPAD; i += tc2::THREADS) s_colexp[i] = 0;
    __syncthreads();

    // ---- B planes: the output columns of Q, split per column (as k_basis_tc) ----
    auto qval = [&](int k, int i) -> double {
        if (i > nev || k >= m) return 0.0;
        if (i < nev && k > i + np) return 0.0;
        return Q[k + (size_t)i * m];
    };
    const int kg = kpad >> 3;
    for (int it = tid; it < NPAD * kg; it += tc2::THREADS) {
        const int i = it / kg, g = it % kg;
        int emax = 0;
        for (int e = 0; e < 8; ++e) emax = max(emax, exp_field(qval(8 * g + e, i)));
        atomicMax(&s_colexp[i], emax);
    }
    __syncthreads();
    const size_t bplane = (size_t)NPAD * kpad * 2;
    for (int it = tid; it < NPAD * kg; it += tc2::THREADS) {
        const int i = it / kg, g = it % kg;
        double x[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) x[e] = qval(8 * g + e, i);
        uint4 pl[NDIG];
        split8(x, s_colexp[i], pl);
        const uint32_t off = kmajor_off(i, 8 * g, kpad);
#pragma unroll
        for (int q = 0; q < NDIG; ++q) *reinterpret_cast<uint4 *>(sB + q * bplane + off) = pl[q];
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    const uint32_t taddr = s_taddr;
    double nrm = 0.0;

    // Waits are taken by lane 0 and broadcast, so a warp's lanes always agree
    // on whether to go on (a failed wait then exits the whole warp's loop).
    auto wait0 = [&](uint64_t *bar, uint32_t par) -> bool {
        int ok = 1;
        if (lane == 0) ok = mbar_wait_bounded(bar, par, limit, fail) ? 1 : 0;
        return __shfl_sync(0xffffffffu, ok, 0) != 0;
    };
    if (warp == tc2::CTRL_WARP) {
        // ---------------- bulk copies (whole warp) and MMAs (lane 0) ----------------
        if (lane == 0) fence_after();
        int loads = 0;                          // blocks whose copies were issued
        auto issue_load = [&](int b) {
            const int R0 = t.row0 + b * BM;
            const int rows = min(BM, ((t.row1 - R0) + 1) & ~1);   // even: 16-byte multiple
            const uint32_t bytes = (uint32_t)rows * 8u;
            if (lane == 0) mbar_expect_tx(&bar_full, bytes * (uint32_t)m);
            __syncwarp();
            for (int k = lane; k < m; k += 32)
                bulk_g2s(stage + (size_t)k * BM, P.V + R0 + (size_t)k * ld, bytes, &bar_full);
            loads = b + 1;
        };
        const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
        const uint32_t sboB = (uint32_t)kg * 128u, sboA = (uint32_t)(tc2::KH / 8) * 128u;
        auto mma_half = [&](int hh, uint32_t dacc) {
            const int k0 = 2 * hh, k1 = min(ksteps, 2 * hh + 2);
            for (int q = 0; q < NDIG; ++q) {
                const uint32_t id = instr_desc(BM, (NDIG - q) * NPAD);
                const uint32_t d = dacc + (uint32_t)(q * NPAD);
                for (int kk = k0; kk < k1; ++kk) {
                    const uint64_t ad = smem_desc(a0 + (uint32_t)(hh * tc2::ABUF + q * tc2::APLANE) +
                                                      (uint32_t)(kk - k0) * 256u, 128u, sboA);
                    mma(d, ad, smem_desc(b0 + (uint32_t)kk * 256u, 128u, sboB), id, (q | kk) ? 1u : 0u);
                }
            }
        };
        issue_load(0);
        for (int b = 0; b < nblk; ++b) {
            const int ab = b & 1;
            const uint32_t dacc = taddr + (uint32_t)ab * ACC;
            if (b >= 2 && !wait0(&bar_accempty[ab], (uint32_t)(((b >> 1) - 1) & 1))) break;
            if (!wait0(&bar_afull[0], (uint32_t)(b & 1))) break;
            if (lane == 0) {
                fence_after();
                mma_half(0, dacc);
                mma_commit(&bar_aempty[0]);
            }
            __syncwarp();
            if (b + 1 < nblk) {                 // stage released after the first half's split
                if (!wait0(&bar_empty, (uint32_t)(b & 1))) break;
                issue_load(b + 1);
            }
            if (two && !wait0(&bar_afull[1], (uint32_t)(b & 1))) break;
            if (lane == 0) {
                if (two) {
                    fence_after();
                    mma_half(1, dacc);
                    mma_commit(&bar_aempty[1]);
                }
                mma_commit(&bar_accfull[ab]);
            }
            __syncwarp();
        }
        // drain: the MMAs issued so far, then the last bulk copy issued
        if (lane == 0) {
            mma_commit(&bar_drain);
            for (unsigned spins = 0; spins < (unsigned)WAIT_LIMIT_DEFAULT; ++spins)
                if (mbar_try_wait(&bar_drain, 0u)) break;
            if (loads > 0)
                for (unsigned spins = 0; spins < (unsigned)WAIT_LIMIT_DEFAULT; ++spins)
                    if (mbar_try_wait(&bar_full, (uint32_t)((loads - 1) & 1))) break;
        }
        __syncwarp();
    } else if (warp < tc2::SPLIT_WARPS) {
        // ---------------- splitters: two threads per row ----------------
        const int row = tid >> 1, part = tid & 1;
        for (int b = 0; b < nblk; ++b) {
            const bool rok = t.row0 + b * BM + row < t.row1;
            if (!wait0(&bar_full, (uint32_t)(b & 1))) break;
            // exponent of the row; the second half's values stay in registers
            double x1[2][8];
            int emax = 0;
#pragma unroll
            for (int g = 0; g < 2; ++g)
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int k0 = part * 16 + g * 8 + e, k1 = tc2::KH + k0;
                    const double v0 = (rok && k0 < m) ? stage[(size_t)k0 * BM + row] : 0.0;
                    x1[g][e] = (rok && k1 < m) ? stage[(size_t)k1 * BM + row] : 0.0;
                    emax = max(emax, max(exp_field(v0), exp_field(x1[g][e])));
                }
            emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 1));
            if (part == 0) s_rowexp[b & 3][row] = emax;
            // first half, from the stage
            if (b >= 1 && !wait0(&bar_aempty[0], (uint32_t)((b - 1) & 1))) break;
#pragma unroll
            for (int g = 0; g < 2; ++g) {
                double x0[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int k0 = part * 16 + g * 8 + e;
                    x0[e] = (rok && k0 < m) ? stage[(size_t)k0 * BM + row] : 0.0;
                }
                split8_store(x0, emax, sA, kmajor_off(row, part * 16 + g * 8, tc2::KH));
            }
            fence_async_smem();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&bar_afull[0]);
                mbar_arrive(&bar_empty);
            }
            // second half, from registers (ncv <= 32: none)
            if (!two) continue;
            if (b >= 1 && !wait0(&bar_aempty[1], (uint32_t)((b - 1) & 1))) break;
#pragma unroll
            for (int g = 0; g < 2; ++g)
                split8_store(x1[g], emax, sA + tc2::ABUF, kmajor_off(row, part * 16 + g * 8, tc2::KH));
            fence_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&bar_afull[1]);
        }
    } else {
        // ---------------- recombiners ----------------
        const int q4 = warp & 3, oh = (warp - tc2::SPLIT_WARPS) >> 2;
        const int r = 32 * q4 + lane;
        const double hn = h[nev];
        const double qlast = Q[(m - 1) + (size_t)(nev - 1) * m];
        const double *__restrict__ rin = (m & 1) ? P.r1 : P.r0;
        double *__restrict__ rout = (nev & 1) ? P.r1 : P.r0;
        for (int b = 0; b < nblk; ++b) {
            const int ab = b & 1;
            if (!wait0(&bar_accfull[ab], (uint32_t)((b >> 1) & 1))) break;
            fence_after();
            const int orow = t.row0 + b * BM + r;
            const bool ok = orow < t.row1;
            const int exr = s_rowexp[b & 3][r];
            const uint32_t lane_base = taddr + ((uint32_t)(32 * q4) << 16) + (uint32_t)ab * ACC;
            for (int c0 = 4 * oh; c0 < nout; c0 += 8) {
                float d[NDIG][4];
                tmem_ld_levels4(lane_base + (uint32_t)c0, (uint32_t)NPAD, d);
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int i = c0 + e;
                    if (i >= nout || !ok) continue;
                    float lv[NDIG];
#pragma unroll
                    for (int L = 0; L < NDIG; ++L) lv[L] = d[L][e];
                    const double v = combine(lv, exr, s_colexp[i]);
                    if (i < nev) {
                        P.V[orow + (size_t)i * ld] = v;
                        P.V32[orow + (size_t)i * ld] = (float)v;
                    } else {                                      // residual (HLanc.hpp:1605-1614)
                        double res = rin[orow] * qlast;
                        if (hn > 0.0) res = res + hn * v;
                        rout[orow] = res;
                        nrm = fma(res, res, nrm);
                    }
                }
            }
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&bar_accempty[ab]);
        }
    }

    // release tensor memory: the MMAs are drained (above) and every TMEM read
    // completed before its accempty arrival
    fence_before();
    __syncthreads();
    if (warp == tc2::CTRL_WARP) {
        fence_after();
        tmem_dealloc(taddr, NCOLS);
    }
    if (*fail && tid == 0) atomicExch(&S->err, DEV_ERR_MMA_WAIT);
    nrm = block_sum0(nrm, s_red);
    if (tid == 0) s_mine[0] = nrm;
    __syncthreads();
    if (!finish_tile(P, blockIdx.x - P.tile0, 1, s_mine, s_tot)) return;
    if (tid == 0) {
        S->rnorm = sqrt(s_tot[0]);                    // HLanc.hpp:1735
        S->phase = PH_EXTEND;
        S->sumnev += nev;
        S->napply += 1;
    }
}

template <int NPAD>
static void basis_tc2_t(const Problem *P_d, const Tile *tiles_d, int ntiles, cudaStream_t s) {
    static std::atomic<unsigned long long> attr{0};
    const size_t smem = basis_tc2_smem<NPAD>();
    smem_limit_once(k_basis_tc2<NPAD>, (int)smem, attr);
    prof_begin(s);
    k_basis_tc2<NPAD><<<ntiles, tc2::THREADS, smem, s>>>(P_d, tiles_d);
    prof_end(KC_BASIS, s);
    launch_counter() += 1;
    variant_counter(HLANC_KL_BASIS_TC) += 1;
}

template <int NPAD>
static size_t basis_tc_smem() {
    return (size_t)tc::NDIG * tc::BM * tc::KMAX * 2 + (size_t)tc::NDIG * NPAD * tc::KMAX * 2;
}

template <int NPAD>
static void basis_tc_t(const Problem *P_d, const Tile *tiles_d, int ntiles, cudaStream_t s) {
    static std::atomic<unsigned long long> attr{0};
    const size_t smem = basis_tc_smem<NPAD>();
    smem_limit_once(k_basis_tc<NPAD, false>, (int)smem, attr);
    prof_begin(s);
    k_basis_tc<NPAD, false><<<ntiles, tc::THREADS, smem, s>>>(P_d, tiles_d);
    prof_end(KC_BASIS, s);
    launch_counter() += 1;
    variant_counter(HLANC_KL_BASIS_TC) += 1;
}

// The tensor-core basis update serves problems with ncv <= 64 and
// nev + 1 <= 64 (nev_max is the engine's bucket of the adjusted nev: 4, 8,
// ..., 40, 48, 56 or 63); the caller uses k_basis otherwise.
bool basis_tc_fits(int max_ncv, int nev_max) { return max_ncv <= tc::KMAX && nev_max + 1 <= tc::NMAX; }

// Up to 32 outputs the warp-specialised kernel (two accumulators fit the
// 512 TMEM columns); 33..64 outputs the one-phase-at-a-time kernel.
void launch_basis_tc(const Problem *P_d, const Tile *tiles_d, int ntiles, int nev_max, cudaStream_t s) {
    const int nout = nev_max + 1;
    if (nout <= 16) basis_tc2_t<16>(P_d, tiles_d, ntiles, s);
    else if (nout <= 32) basis_tc2_t<32>(P_d, tiles_d, ntiles, s);
    else if (nout <= 48) basis_tc_t<48>(P_d, tiles_d, ntiles, s);
    else basis_tc_t<64>(P_d, tiles_d, ntiles, s);
}

// Ritz vectors of the converged problems on the tensor cores (ncv <= 64).
// One shape serves every ncv: the kernel is bound by splitting V, whose
// cost does not depend on the padded output count.  Measured on GB300
// (4.1M rows, ncv 60): 3.2 ms, against 25.3 ms for the FP64 kernel k_ritz.
bool ritz_tc_fits(int max_ncv) { return max_ncv <= tc::NMAX && max_ncv <= tc::KMAX; }

void launch_ritz_tc(const Problem *P_d, const Tile *tiles_d, int ntiles, cudaStream_t s) {
    static std::atomic<unsigned long long> attr{0};
    const size_t smem = basis_tc_smem<64>();
    smem_limit_once(k_basis_tc<64, true>, (int)smem, attr);
    prof_begin(s);
    k_basis_tc<64, true><<<ntiles, tc::THREADS, smem, s>>>(P_d, tiles_d);
    prof_end(KC_RITZ, s);
    launch_counter() += 1;
    variant_counter(HLANC_KL_RITZ_TC) += 1;
}


}  // namespace hlanc
