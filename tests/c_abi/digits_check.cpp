// Host build of the slicer's digit arithmetic (cutc_gb300/csrc/digits.cuh), checked
// against exact arithmetic:
//   * scaled_round on FP64 values rounds x 2^(F - e) to the nearest integer (ties
//     away from zero): |t - x 2^(F - e)| <= 1/2, checked in long double, where
//     the power-of-two scaling is exact;
//   * scaled_round_df on a normalised double-float (hi, lo) gives the same t as
//     scaled_round on hi + lo whenever that sum is exact in FP64, on random values
//     over a wide exponent range, on exact ties and on the largest value of a row;
//   * digits_int cuts t into digits with t = sum_s q_s 2^(9 (S - 1 - s)),
//     q_s in [-256, 255] for s > 0 and |q_0| <= 256;
//   * digits_df_fp32 cuts the double-float (hi, lo) in FP32 into integer digits
//     q_s in [-256, 256] whose value sum_s q_s 2^(9 (S - 1 - s)) is within
//     1/2 + 2^-16 of (hi + lo) 2^(F - e) (checked in long double), i.e. within one
//     of scaled_round_df's t.
// Prints "ok <cases> <double-float cases>" and exits 0, or reports the first failure
// and exits 1.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "digits.cuh"

using namespace cutc::digits;

// The exact integer rounding of a normalised double-float hi + lo at the last digit,
// in 64-bit integer arithmetic: the reference the FP32 digit cut is checked against
// (the G slicer used it before the FP32 cut replaced it).
// t for the exact sum x = hi + lo of a normalised double-float (|lo| <= ulp(hi)/2),
// with no FP64 arithmetic: GB300 converts and adds FP64 at 1/64 of its FP32 rate,
// which made the G slicer FP64-bound.  With V = |x| 2^(F - e) = A 2^-Q + B 2^-Q,
// A = |hi| 2^(F - e + Q) an integer and B the signed part of lo,
// floor(V 2^Q) = A + floor(B) and, as 2^(Q-1) is an integer,
// floor(V + 1/2) = (floor(V 2^Q) + 2^(Q-1)) >> Q.
template <int S>
static long long scaled_round_df(float hi, float lo, int e)
{
    constexpr int F = 8 + 9 * (S - 1);
    const unsigned hb = float_bits(hi), lb = float_bits(lo);
    if ((hb & 0x7fffffffu) == 0u)
        return 0;  // lo is zero too
    const unsigned hexp = (hb >> 23) & 0xffu;
    const unsigned long long mh = hexp ? ((hb & 0x7fffffu) | 0x800000u) : (hb & 0x7fffffu);
    const int a = (hexp ? (int)hexp : 1) - 150 + F - e;  // |hi| 2^(F-e) = mh 2^a, a <= F - 23
    const int Q = a < -1 ? -a : 1;
    if (Q >= 26)
        return 0;  // V < 2^(24 - Q) (1 + 2^-24) < 1/2
    const unsigned long long A = mh << (a + Q);
    long long fb = 0;
    if ((lb & 0x7fffffffu) != 0u) {
        const unsigned lexp = (lb >> 23) & 0xffu;
        const unsigned long long ml = lexp ? ((lb & 0x7fffffu) | 0x800000u) : (lb & 0x7fffffu);
        const int sh = (lexp ? (int)lexp : 1) - 150 + F - e + Q;  // |lo| 2^(F-e+Q) = ml 2^sh
        const bool same = ((hb ^ lb) >> 31) == 0u;
        if (sh >= 0) {  // not reached for a normalised pair (sh < 0)
            const long long v = (long long)(ml << (sh < 39 ? sh : 39));
            fb = same ? v : -v;
        } else {
            const int k = -sh;
            if (same)
                fb = k >= 64 ? 0 : (long long)(ml >> k);
            else
                fb = k >= 64 ? -1 : -(long long)((ml + (1ull << k) - 1) >> k);
        }
    }
    const unsigned long long T = A + (unsigned long long)fb;  // the true sum is in [0, 2^64)
    const long long r = (long long)((T + (1ull << (Q - 1))) >> Q);
    return (hb >> 31) ? -r : r;
}


static unsigned long long rng_state = 0x9e3779b97f4a7c15ull;
static unsigned long long next_u64()
{
    rng_state ^= rng_state << 13;
    rng_state ^= rng_state >> 7;
    rng_state ^= rng_state << 17;
    return rng_state;
}
static double uniform() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }

static long cases = 0, df_cases = 0;

static void fail(const char *what, int S, double x, float hi, float lo, int e, long long a,
                 long long b)
{
    std::printf("FAIL %s S=%d x=%.17g hi=%.9g lo=%.9g e=%d got=%lld want=%lld\n", what, S, x,
                (double)hi, (double)lo, e, a, b);
    std::exit(1);
}

template <int S>
static void check_fp32_digits(float hi, float lo, int e, double x)
{
    constexpr int F = 8 + 9 * (S - 1);
    float q[S];
    digits_df_fp32<S>(hi, lo, e, q);
    long long back = 0;
    for (int s = 0; s < S; s++) {
        if (q[s] != std::rint(q[s]) || q[s] < -256.0f || q[s] > 256.0f)
            fail("fp32 digit", S, x, hi, lo, e, (long long)q[s], s);
        back = back * 512 + (long long)q[s];
    }
    const long double v = std::ldexp((long double)x, F - e);
    if (std::fabs((double)((long double)back - v)) > 0.5 + std::ldexp(1.0, -16))
        fail("fp32 digits value", S, x, hi, lo, e, back, 0);
}

template <int S>
static void check_value(double x, int e)
{
    constexpr int F = 8 + 9 * (S - 1);
    const long long t = scaled_round<S>(x, e);
    // rounding of x 2^(F - e): within 1/2, ties away from zero
    const long double v = std::ldexp((long double)x, F - e);
    const long double d = (long double)t - v;
    if (std::fabs((double)d) > 0.5 ||
        (std::fabs((double)d) == 0.5 && std::fabs((double)t) < std::fabs((double)v)))
        fail("scaled_round", S, x, 0.f, 0.f, e, t, 0);
    // digits
    int q[S];
    digits_int<S>(t, q);
    long long back = 0;
    for (int s = 0; s < S; s++) {
        if (s > 0 && (q[s] < -256 || q[s] > 255))
            fail("digit range", S, x, 0.f, 0.f, e, q[s], s);
        back = back * 512 + q[s];
    }
    if (back != t || q[0] < -256 || q[0] > 256)
        fail("digits", S, x, 0.f, 0.f, e, back, t);
    // the double-float path on the same value, when x splits exactly into (hi, lo)
    const float hi = (float)x;
    const float lo = (float)(x - (double)hi);
    if ((double)hi + (double)lo == x && (double)lo == x - (double)hi) {
        const long long u = scaled_round_df<S>(hi, lo, e);
        if (u != t)
            fail("scaled_round_df", S, x, hi, lo, e, u, t);
        check_fp32_digits<S>(hi, lo, e, x);
        df_cases++;
    }
    cases++;
}

// exponent e with |x| < 2^e
static int row_exp(double x)
{
    int ex;
    std::frexp(x, &ex);  // |x| in [2^(ex-1), 2^ex)
    return ex;
}

template <int S>
static void run()
{
    constexpr int F = 8 + 9 * (S - 1);
    for (int i = 0; i < 200000; i++) {
        // values over a wide range, 24 to 53 significant bits, rows whose maximum is up
        // to 2^40 larger
        double x = (2.0 * uniform() - 1.0) * std::ldexp(1.0, (int)(next_u64() % 120) - 60);
        if (i % 3 == 0)
            x = (double)(float)x + std::ldexp((double)(float)x, -24) * (uniform() - 0.5);
        if (x == 0.0)
            continue;
        const int e = row_exp(x) + (int)(next_u64() % 41);
        check_value<S>(x, e);
        check_value<S>(-x, e);
    }
    for (int i = 0; i < 50000; i++) {
        // exact ties: (m + 1/2) 2^(e - F)
        const int e = (int)(next_u64() % 80) - 40;
        const long long m = (long long)(next_u64() % (1ull << 30));
        const double x = std::ldexp((double)m + 0.5, e - F);
        if (std::fabs(x) >= std::ldexp(1.0, e))
            continue;
        check_value<S>(x, e);
        check_value<S>(-x, e);
    }
    // rows at the ends of the FP32 range: 2^(8 - e) outside [2^-126, 2^127] (the FP32
    // cut scales in two steps), subnormal hi
    for (int i = 0; i < 20000; i++) {
        const int ex = (i & 1) ? 100 + (int)(next_u64() % 27) : -149 + (int)(next_u64() % 40);
        double x = (2.0 * uniform() - 1.0) * std::ldexp(1.0, ex);
        x = (double)(float)x;  // exactly one float, lo = 0
        if (x == 0.0)
            continue;
        const int e = row_exp(x) + (int)(next_u64() % 3);
        check_value<S>(x, e);
    }
    // the row maximum itself and values just below a power of two
    for (int k = -30; k <= 30; k++) {
        const double x = std::nextafter(std::ldexp(1.0, k), 0.0);
        check_value<S>(x, k);
        check_value<S>(std::ldexp(1.0, k - 1), k);
    }
}

int main()
{
    run<3>();
    run<4>();
    run<5>();
    run<6>();
    run<7>();
    if (df_cases < cases / 10) {
        std::printf("FAIL too few double-float cases: %ld of %ld\n", df_cases, cases);
        return 1;
    }
    std::printf("ok %ld %ld\n", cases, df_cases);
    return 0;
}
