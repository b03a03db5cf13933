// Rounding an operand to its S signed base-2^9 digits: FP64 operands in integer
// arithmetic, double-float operands in FP32 arithmetic (digits_df_fp32).
//
// An operand value x of a row with exponent e (|x| < 2^e) is rounded at its
// last digit, t = sign(x) floor(|x| 2^(F - e) + 1/2) with F = 8 + 9 (S - 1),
// and t is cut into digits q_0 .. q_{S-1} (q_s in [-256, 255] for s > 0) with
// t = sum_s q_s 2^(9 (S - 1 - s)).  Everything here is callable from device code
// (the slicing kernels) and from host code, where a plain C++ build checks it
// against exact arithmetic.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define CUTC_HD __host__ __device__ __forceinline__
#else
#define CUTC_HD inline
#endif

namespace cutc {
namespace digits {

CUTC_HD unsigned float_bits(float x)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    unsigned u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}

CUTC_HD unsigned long long double_bits(double x)
{
#if defined(__CUDA_ARCH__)
    return (unsigned long long)__double_as_longlong(x);
#else
    unsigned long long u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}

// t for an FP64 value x
template <int S>
CUTC_HD long long scaled_round(double x, int e)
{
    constexpr int F = 8 + 9 * (S - 1);
    const unsigned long long bits = double_bits(x);
    const int E = (int)((bits >> 52) & 0x7ff);
    long long t = 0;
    if (E != 0) {
        const unsigned long long mant = (bits & ((1ull << 52) - 1)) | (1ull << 52);
        const int sh = E - 1075 - e + F;
        unsigned long long T;
        if (sh >= 0)
            T = mant << sh;  // < 2^F because |x| < 2^e
        else if (sh > -64)
            T = (mant + (1ull << (-sh - 1))) >> (-sh);
        else
            T = 0;
        t = (bits >> 63) ? -(long long)T : (long long)T;
    }
    return t;
}

// IEEE FP32 operations, rounded to nearest, never contracted into FMAs (host builds of
// this header take -ffp-contract=off)
CUTC_HD float f_add(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}

CUTC_HD float f_mul(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}

CUTC_HD float f_rint(float a)  // nearest integer, ties to even
{
#if defined(__CUDA_ARCH__)
    return rintf(a);
#else
    return __builtin_rintf(a);
#endif
}

CUTC_HD float pow2_float(int k)  // 2^k for k in [-126, 127]
{
    const unsigned u = (unsigned)(k + 127) << 23;
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, sizeof f);
    return f;
#endif
}

// The S digits of the normalised double-float hi + lo (|lo| <= ulp(hi)/2) of a row with
// exponent e (|hi + lo| < 2^e), cut in FP32 arithmetic on the FMA pipe instead of the
// 64-bit integer work of an exact rounding followed by digits_int, which kept the
// integer pipe busy.
// With v = (hi + lo) 2^(8 - e) held as the pair (xh, xl), |v| < 256:
//   q_s = rint(xh);  (xh, xl) <- TwoSum(xh - q_s, xl) * 2^9
// (xh - q_s is exact, TwoSum is exact, the scaling is exact), so
//   v = sum_{s < S} q_s 2^(-9 s) + r 2^(-9 (S - 1)),  |r| <= 1/2 + |xl| <= 1/2 + 2^-16,
// and every |q_s| <= 256 (the remainder before a scaling is at most 1/2 + 2^-16).  The
// digits are the integers q_s, returned as floats.  Scaling by 2^(8 - e) takes two
// exact steps when 8 - e leaves the FP32 exponent range; values it makes subnormal are
// below 2^-126, where every digit is zero.
template <int S>
CUTC_HD void digits_df_fp32(float hi, float lo, int e, float (&q)[S])
{
    const int k = 8 - e;  // -119 <= k <= 157 for FP32 hi and lo
    const int k1 = k / 2, k2 = k - k1;
    const float c1 = pow2_float(k1), c2 = pow2_float(k2);
    float xh = f_mul(f_mul(hi, c1), c2), xl = f_mul(f_mul(lo, c1), c2);
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int s = 0; s < S; s++) {
        const float d = f_rint(xh);
        q[s] = d;
        if (s == S - 1)
            break;
        const float a = f_add(xh, -d);
        const float sm = f_add(a, xl);
        const float bb = f_add(sm, -a);
        const float er = f_add(f_add(a, -f_add(sm, -bb)), f_add(xl, -bb));
        xh = f_mul(sm, 512.0f);
        xl = f_mul(er, 512.0f);
    }
}

// q_0 .. q_{S-1} of t
template <int S>
CUTC_HD void digits_int(long long t, int (&q)[S])
{
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int s = S - 1; s >= 1; s--) {
        const long long d = ((t + 256) & 511) - 256;
        q[s] = (int)d;
        t = (t - d) >> 9;
    }
    q[0] = (int)t;
}

}  // namespace digits
}  // namespace cutc
