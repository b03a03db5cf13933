// Double-float ("df") arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers with |lo| <= ulp(hi)/2, carrying ~48 significant bits.  Built
// from the error-free transformations of Dekker (1971) and Knuth (TwoSum), with
// the FMA form of TwoProd, as organised in Hida, Li & Bailey's QD library
// (2001).  Used on GB300 for the pair terms, because FP32 issues at 64x the
// FP64 rate there while FP64-level accuracy (~1e-14) is still needed.
#pragma once

#include <cuda_runtime.h>

namespace cutc {
namespace df {

struct D {
    float hi, lo;
};

__device__ __forceinline__ D make(float h, float l) { return D{h, l}; }

__device__ __forceinline__ D from_double(double x)
{
    const float h = __double2float_rn(x);
    const float l = __double2float_rn(x - (double)h);
    return D{h, l};
}

__device__ __forceinline__ double to_double(D a) { return (double)a.hi + (double)a.lo; }

// s + e = a + b exactly (Knuth TwoSum)
__device__ __forceinline__ D two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return D{s, e};
}

// s + e = a + b exactly, requires |a| >= |b| (Dekker FastTwoSum)
__device__ __forceinline__ D fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return D{s, e};
}

// p + e = a * b exactly (FMA TwoProd)
__device__ __forceinline__ D two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    return D{p, e};
}

__device__ __forceinline__ D add(D a, D b)
{
    D s = two_sum(a.hi, b.hi);
    D t = two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ D neg(D a) { return D{-a.hi, -a.lo}; }

__device__ __forceinline__ D sub(D a, D b) { return add(a, neg(b)); }

__device__ __forceinline__ D add_f(D a, float b)
{
    D s = two_sum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ D mul(D a, D b)
{
    D p = two_prod(a.hi, b.hi);
    p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
    p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
    return fast_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ D mul_f(D a, float b)
{
    D p = two_prod(a.hi, b);
    p.lo = __fmaf_rn(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}

// a * b + c, with one renormalisation
__device__ __forceinline__ D fma(D a, D b, D c)
{
    D p = two_prod(a.hi, b.hi);
    p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
    p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
    D s = two_sum(p.hi, c.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(p.lo, c.lo));
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ D sqr(D a)
{
    D p = two_prod(a.hi, a.hi);
    p.lo = __fmaf_rn(2.0f * a.hi, a.lo, p.lo);
    return fast_two_sum(p.hi, p.lo);
}

// 1 / b: FP32 reciprocal refined by one Newton step in df arithmetic
__device__ __forceinline__ D recip(D b)
{
    const float x = __frcp_rn(b.hi);
    // r = 1 - b x  (exact enough in df), y = x + x r
    D bx = mul_f(b, x);
    D r = add_f(neg(bx), 1.0f);
    D y = add_f(mul_f(r, x), x);
    return y;
}

// sqrt(a) for a > 0: FP32 sqrt refined by one Newton step in df arithmetic
__device__ __forceinline__ D sqrt(D a)
{
    const float x = __fsqrt_rn(a.hi);
    // y = x + (a - x^2) / (2x)
    D x2 = two_prod(x, x);
    D r = sub(a, x2);
    const float corr = __fdiv_rn(r.hi, 2.0f * x);
    return fast_two_sum(x, corr);
}

}  // namespace df
}  // namespace cutc
