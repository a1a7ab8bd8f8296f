// fixed_point.cuh -- exact fixed-point products of FP64 values on the
// integer pipes (used by the hybrid CGS kernels).
//
// GB300 retires one FP64 FMA per SM sub-partition every 64 cycles, and a CGS
// pass needs one FMA per 8-byte element, so FP64 alone cannot keep up with
// HBM.  The CGS kernels therefore run about half of every column panel on
// the integer pipes, which work concurrently with the FP64 pipe.
//
// A double x with |x| < 2^(E+1) becomes X = round(x * 2^(57-E)), |X| < 2^58,
// held as two signed limbs X = x1 * 2^29 + x0 (|x1|, |x0| < 2^29, both
// carrying the sign of x).  The product of two such values is four
// 32x32 -> 64-bit multiply-adds into three 64-bit accumulators (units
// 2^58, 2^29, 1).  Sums are exact integers up to the one final conversion
// to FP64, so the error is the quantisation of the two inputs: at most
// 2^-58 of each factor's scale 2^(E+1).  Two rules keep the sums exact:
//  - every limb product is below 2^58 in magnitude and the middle
//    accumulator takes two per step, so fx_carry must run at least every
//    FX_MACS = 16 steps;
//  - the top accumulator is never carried out, so the sum of |X * Y| over
//    all steps before fx_to_double must stay below 2^120.  For the CGS
//    kernels this follows from the orthonormal basis (Cauchy-Schwarz): a
//    column's entries in the <= 256 rows a thread visits (tiles are capped
//    at 65,536 rows) and a row's entries in the <= 128 columns have
//    sum |v| <= 16 and sum |v| <= 11.4, with |X| <= 2^57 |v| and |Y| < 2^58.
//
// rsc = 1027 + E.  Lanczos basis vectors are unit vectors, so their entries
// use E = 0 (FX_RS_UNIT).  Zeros and subnormals give X = 0.
//
// The functions also compile as plain C++ so that the host tests can check
// them against 128-bit integer arithmetic.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define FX_HD __host__ __device__ __forceinline__
#else
#define FX_HD inline
#endif

namespace hlanc {

constexpr int FX_RS_UNIT = 1027;
constexpr int FX_MACS = 16;          // multiply-add steps between carries

FX_HD unsigned long long fx_bits(double x) {
#if defined(__CUDA_ARCH__)
    return (unsigned long long)__double_as_longlong(x);
#else
    unsigned long long b;
    memcpy(&b, &x, sizeof b);
    return b;
#endif
}

FX_HD double fx_from_bits(unsigned long long b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, sizeof x);
    return x;
#endif
}

// high word of (hi:lo) << s, 0 <= s < 32
FX_HD unsigned fx_funnel_l(unsigned lo, unsigned hi, unsigned s) {
#if defined(__CUDA_ARCH__)
    return __funnelshift_l(lo, hi, s);
#else
    return (unsigned)(((((unsigned long long)hi << 32) | lo) << (s & 31u)) >> 32);
#endif
}

FX_HD int fx_clz64(unsigned long long x) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

// E for a set of doubles whose largest |high word| is max_hi_word (the
// clamp keeps rsc - 0 above 63, so zeros still map to 0)
FX_HD int fx_scale(unsigned max_hi_word) {
    const int e = (int)(max_hi_word >> 20) - 1023;
    return e > -960 ? e : -960;
}

FX_HD unsigned fx_hi_abs(double x) { return (unsigned)(fx_bits(x) >> 32) & 0x7FFFFFFFu; }

FX_HD void fx_split(double x, int rsc, int &x1, int &x0) {
    const unsigned long long b = fx_bits(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7FFu);
    // significand with its leading one at bit 62
    const unsigned mh = (fx_funnel_l(lo, hi, 10) & 0x3FFFFFFFu) | 0x40000000u;
    const unsigned long long mt = ((unsigned long long)mh << 32) | (unsigned long long)(lo << 10);
    const unsigned d = (unsigned)(rsc - e);
    const unsigned sh = d < 63u ? d : 63u;                  // >= 4 when |x| < 2^(E+1)
    const unsigned long long q = (mt >> sh) + 1ull;          // X * 2 + 1: round to nearest
    int a1 = (int)(q >> 30);
    int a0 = (int)((unsigned)(q >> 1) & 0x1FFFFFFFu);
    if ((int)hi < 0) {
        a1 = -a1;
        a0 = -a0;
    }
    x1 = a1;
    x0 = a0;
}

struct FxAcc {
    long long a2, a1, a0;   // value = a2 * 2^58 + a1 * 2^29 + a0
};

FX_HD void fx_zero(FxAcc &A) { A.a2 = A.a1 = A.a0 = 0; }

FX_HD void fx_mac(FxAcc &A, int x1, int x0, int y1, int y0) {
    A.a2 += (long long)x1 * y1;
    A.a1 += (long long)x1 * y0;
    A.a1 += (long long)x0 * y1;
    A.a0 += (long long)x0 * y0;
}

// Move the carries up: afterwards 0 <= a1, a0 < 2^29.
FX_HD void fx_carry(FxAcc &A) {
    A.a1 += A.a0 >> 29;
    A.a0 &= 0x1FFFFFFFll;
    A.a2 += A.a1 >> 29;
    A.a1 &= 0x1FFFFFFFll;
}

// value * 2^e2 rounded to the nearest double (ties away from zero); values
// below the normal range give 0.
FX_HD double fx_to_double(FxAcc A, int e2) {
    fx_carry(A);
    const unsigned long long low = ((unsigned long long)A.a1 << 29) | (unsigned long long)A.a0;   // < 2^58
    const long long shi = A.a2 >> 6;                                    // 128-bit two's complement
    unsigned long long h = (unsigned long long)shi;
    unsigned long long l = ((unsigned long long)A.a2 << 58) | low;
    const bool neg = shi < 0;
    if (neg) {
        l = ~l + 1ull;
        h = ~h + (l == 0ull ? 1ull : 0ull);
    }
    if ((h | l) == 0ull) return 0.0;
    const int lz = h ? fx_clz64(h) : 64 + fx_clz64(l);
    unsigned long long top;
    if (lz >= 64) top = l << (lz - 64);
    else if (lz == 0) top = h;
    else top = (h << lz) | (l >> (64 - lz));
    const long long be = (long long)(127 - lz) + e2 + 1023;
    if (be <= 0) return 0.0;
    const unsigned long long bits = ((unsigned long long)(be - 1) << 52) + ((top + (1ull << 10)) >> 11);
    const double r = fx_from_bits(bits);
    return neg ? -r : r;
}

}  // namespace hlanc
