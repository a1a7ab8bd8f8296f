// Host check of the fixed-point helpers of the hybrid CGS kernels
// (hlanc_gb300/csrc/fixed_point.cuh) against 128-bit integer arithmetic.
// Build: g++ -O2 -std=c++17 fixed_point_test.cpp; exit status 0 = pass.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../hlanc_gb300/csrc/fixed_point.cuh"

using namespace hlanc;
typedef __int128 i128;

static unsigned long long g_rng = 0x9E3779B97F4A7C15ull;
static unsigned long long next64() {
    g_rng ^= g_rng << 13;
    g_rng ^= g_rng >> 7;
    g_rng ^= g_rng << 17;
    return g_rng;
}
static double uni() { return (double)(next64() >> 11) * 0x1.0p-53; }   // [0, 1)

static int failures = 0;
#define CHECK(cond, ...)                              \
    do {                                              \
        if (!(cond)) {                                \
            if (failures < 20) printf(__VA_ARGS__);   \
            ++failures;                               \
        }                                             \
    } while (0)

static i128 fx_value(int x1, int x0) { return (i128)x1 * ((i128)1 << 29) + x0; }

// exact value of an accumulator
static i128 acc_value(const FxAcc &A) {
    return (i128)A.a2 * ((i128)1 << 58) + (i128)A.a1 * ((i128)1 << 29) + (i128)A.a0;
}

// i128 * 2^e2 as long double (exact enough: 64-bit mantissa), for the rounding check
static long double i128_ld(i128 v, int e2) {
    const bool neg = v < 0;
    unsigned __int128 u = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
    long double hi = (long double)(unsigned long long)(u >> 64), lo = (long double)(unsigned long long)u;
    long double r = ldexpl(hi, 64 + e2) + ldexpl(lo, e2);
    return neg ? -r : r;
}

static double random_value(int E) {
    // magnitudes spread over 70 binades below 2^(E+1), both signs, some exact zeros
    const unsigned long long r = next64();
    if (r % 97 == 0) return 0.0;
    double x = (uni() * 2.0 - 1.0) * ldexp(1.0, E + 1);
    if (r % 5 == 0) x = ldexp(x, -(int)(uni() * 70));
    if (r % 31 == 0) x = std::nextafter(ldexp(1.0, E + 1), 0.0) * ((r & 1) ? 1 : -1);   // largest allowed
    return x;
}

int main() {
    // 1. split: |X - x 2^(57-E)| <= 1/2, limbs below 2^29, sign carried by both limbs
    for (int t = 0; t < 1000000; ++t) {
        const int E = (int)(uni() * 200) - 100;
        const double x = random_value(E);
        int x1, x0;
        fx_split(x, 1027 + E, x1, x0);
        const long double want = ldexpl((long double)x, 57 - E);
        const long double got = (long double)x1 * 536870912.0L + (long double)x0;
        CHECK(fabsl(got - want) <= 0.5L, "split x=%a E=%d got %.3Lf want %.3Lf\n", x, E, got, want);
        CHECK(std::abs(x1) < (1 << 29) && std::abs(x0) < (1 << 29), "limb range x=%a\n", x);
        CHECK((x >= 0 && x1 >= 0 && x0 >= 0) || (x <= 0 && x1 <= 0 && x0 <= 0), "limb sign x=%a\n", x);
    }
    // zeros, subnormals and the clamped scale
    {
        int x1, x0;
        fx_split(0.0, 1027 + fx_scale(0u), x1, x0);
        CHECK(x1 == 0 && x0 == 0, "zero\n");
        fx_split(-0.0, FX_RS_UNIT, x1, x0);
        CHECK(x1 == 0 && x0 == 0, "-zero\n");
        fx_split(4.9e-324, FX_RS_UNIT, x1, x0);
        CHECK(x1 == 0 && x0 == 0, "subnormal\n");
        fx_split(1.0, FX_RS_UNIT, x1, x0);
        CHECK(fx_value(x1, x0) == ((i128)1 << 57), "one\n");
        CHECK(fx_scale(fx_hi_abs(3.0)) == 1 && fx_scale(fx_hi_abs(-0.75)) == -1, "scale\n");
    }
    // 2. accumulation is exact (checked in 128-bit integers): random inputs
    //    with carries every FX_MACS steps, and the largest same-sign limbs
    //    (sum |X Y| just below the 2^120 limit after 15 steps)
    for (int trial = 0; trial < 2000; ++trial) {
        const int E = (int)(uni() * 40) - 20;
        const bool worst = trial % 10 == 0;
        const int len = worst ? 15 : 1 + (int)(uni() * 300);
        FxAcc A;
        fx_zero(A);
        i128 exact = 0;
        int steps = 0;
        for (int i = 0; i < len; ++i) {
            int x1, x0, y1, y0;
            if (worst) {
                x1 = y1 = x0 = y0 = (trial % 20 == 0) ? (1 << 29) - 1 : -((1 << 29) - 1);
                y1 = y0 = (1 << 29) - 1;
            } else {
                fx_split(random_value(0), FX_RS_UNIT, x1, x0);
                fx_split(random_value(E), 1027 + E, y1, y0);
            }
            fx_mac(A, x1, x0, y1, y0);
            exact += fx_value(x1, x0) * fx_value(y1, y0);
            if (++steps == FX_MACS) {
                steps = 0;
                fx_carry(A);
            }
            CHECK(acc_value(A) == exact, "accumulation trial %d step %d\n", trial, i);
        }
        // 3. conversion: the double nearest to exact * 2^(E - 114)
        const double d = fx_to_double(A, E - 114);
        const long double want = i128_ld(exact, E - 114);
        const long double err = fabsl((long double)d - want);
        CHECK(err <= fabsl(want) * 0x1.0p-53L, "convert trial %d got %a want %La\n", trial, d, want);
    }
    // 3b. a thread's largest case in the projection: 256 rows of a unit
    //     vector with equal entries 1/16 against |w| at the top of its scale
    {
        FxAcc A;
        fx_zero(A);
        i128 exact = 0;
        for (int i = 0; i < 256; ++i) {
            int x1, x0, y1, y0;
            fx_split((i & 1) ? 0.0625 : 0.0625, FX_RS_UNIT, x1, x0);
            fx_split(std::nextafter(2.0, 0.0), 1027 + 0, y1, y0);
            fx_mac(A, x1, x0, y1, y0);
            exact += fx_value(x1, x0) * fx_value(y1, y0);
            if ((i + 1) % FX_MACS == 0) fx_carry(A);
        }
        CHECK(acc_value(A) == exact, "projection bound case\n");
    }
    // 4. dot products against a compensated FP64 reference: error below
    //    the input quantisation bound n * 2^-58 * (|v| scale 1) * 2^(E+1)
    for (int trial = 0; trial < 200; ++trial) {
        const int n = 1000 + (int)(uni() * 4000);
        const int E = (int)(uni() * 600) - 300;
        std::vector<double> v(n), w(n);
        for (int i = 0; i < n; ++i) {
            v[i] = (uni() * 2 - 1) / sqrt((double)n);
            w[i] = (uni() * 2 - 1) * ldexp(1.0, E);
        }
        unsigned mx = 0;
        for (double x : w) mx = mx > fx_hi_abs(x) ? mx : fx_hi_abs(x);
        const int ew = fx_scale(mx);
        FxAcc A;
        fx_zero(A);
        long double ref = 0.0L;
        for (int i = 0; i < n; ++i) {
            int x1, x0, y1, y0;
            fx_split(v[i], FX_RS_UNIT, x1, x0);
            fx_split(w[i], 1027 + ew, y1, y0);
            fx_mac(A, x1, x0, y1, y0);
            if ((i + 1) % FX_MACS == 0) fx_carry(A);
            ref += (long double)v[i] * (long double)w[i];
        }
        const double d = fx_to_double(A, ew - 114);
        const long double bound = (long double)n * ldexpl(1.0L, ew + 1 - 58) * 2.0L;
        CHECK(fabsl((long double)d - ref) <= bound, "dot trial %d err %Le bound %Le\n", trial,
              fabsl((long double)d - ref), bound);
    }
    // 5. zero and sign of the conversion
    {
        FxAcc A;
        fx_zero(A);
        CHECK(fx_to_double(A, 0) == 0.0, "zero conversion\n");
        fx_mac(A, -3, 0, 1, 0);
        CHECK(fx_to_double(A, -58) == -3.0, "negative conversion %a\n", fx_to_double(A, -58));
    }
    printf(failures ? "FAILED %d\n" : "OK\n", failures);
    return failures ? 1 : 0;
}
