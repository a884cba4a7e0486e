// dfloat.cuh - double-float ("double-FP32") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2),
// about 48 significant bits.  On GB300 a warp instruction on the FP32 pipe
// issues in one cycle where an FP64 one occupies its partition's FP64 pipe
// for 64, so short sequential FP64 algorithms (a small Cholesky, for one)
// run several times faster in this arithmetic.  The building blocks are the
// error-free transformations of Knuth (two-sum), Dekker (fast two-sum) and
// the FMA two-product; the add is the accurate variant that also compensates
// the low parts (so cancellation keeps ~48 bits), the square root and the
// reciprocal take one Newton step from the FP32 result.  All operations use
// explicit round-to-nearest intrinsics so that no contraction changes them.
#pragma once

#include <stdint.h>

#include "fpconv.cuh"

namespace iptgb {

struct dfloat {
    float hi, lo;
};

__device__ __forceinline__ dfloat df_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
    return {s, e};
}

// |a| >= |b| (or a == 0)
__device__ __forceinline__ dfloat df_fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dfloat df_add(dfloat x, dfloat y)
{
    dfloat s = df_two_sum(x.hi, y.hi);
    const dfloat t = df_two_sum(x.lo, y.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = df_fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return df_fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ dfloat df_neg(dfloat x) { return {-x.hi, -x.lo}; }

__device__ __forceinline__ dfloat df_sub(dfloat x, dfloat y) { return df_add(x, df_neg(y)); }

__device__ __forceinline__ dfloat df_mul(dfloat x, dfloat y)
{
    const float p = __fmul_rn(x.hi, y.hi);
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fmaf_rn(x.hi, y.lo, e);
    e = __fmaf_rn(x.lo, y.hi, e);
    return df_fast_two_sum(p, e);
}

// x * y with a plain float y
__device__ __forceinline__ dfloat df_mul_f(dfloat x, float y)
{
    const float p = __fmul_rn(x.hi, y);
    float e = __fmaf_rn(x.hi, y, -p);
    e = __fmaf_rn(x.lo, y, e);
    return df_fast_two_sum(p, e);
}

// sqrt(a) for a > 0: s = sqrt(a.hi), corrected by (a - s^2) / (2 s)
__device__ __forceinline__ dfloat df_sqrt(dfloat a)
{
    const float s = __fsqrt_rn(a.hi);
    const float p = __fmul_rn(s, s);
    const float pe = __fmaf_rn(s, s, -p);
    // a - s^2, the leading part is exact (Sterbenz)
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), a.lo);
    return df_fast_two_sum(s, __fdiv_rn(r, __fmul_rn(2.0f, s)));
}

// 1 / a: y = 1 / a.hi, corrected by y (1 - a y)
__device__ __forceinline__ dfloat df_recip(dfloat a)
{
    const float y = __frcp_rn(a.hi);
    const dfloat ay = df_mul_f(a, y);
    const dfloat one = {1.0f, 0.0f};
    const dfloat e = df_sub(one, ay);
    return df_fast_two_sum(y, __fmul_rn(y, e.hi));
}

// (S, s) += (ah + al)(bh + bl), dropping al bl: the exact two-product of the
// leading parts (p, fma(ah, bh, -p)), the cross terms folded into its error,
// p added to S with an exact two-sum whose error joins s: 12 FP32 operations,
// the accumulation step of the double-float dot products.
__device__ __forceinline__ void df_acc(float &S, float &s, float ah, float al, float bh, float bl)
{
    const float p = __fmul_rn(ah, bh);
    const float pe = __fmaf_rn(ah, bh, -p);
    const float t = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, pe));
    const float u = __fadd_rn(S, p);
    const float bp = __fsub_rn(u, S);
    const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(u, bp)), __fsub_rn(p, bp));
    S = u;
    s = __fadd_rn(s, __fadd_rn(err, t));
}

// |h| = |hi| + sgn(hi) lo added to a double-float sum (S, C) on the FP32 pipe
__device__ __forceinline__ void df_abs_add(float &S, float &C, float hi, float lo)
{
    const float a = fabsf(hi);
    const float bl = hi < 0.0f ? -lo : lo;
    const float t = __fadd_rn(S, a);
    const float bp = __fsub_rn(t, S);
    const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(t, bp)), __fsub_rn(a, bp));
    S = t;
    C = __fadd_rn(C, __fadd_rn(err, bl));
}

// exact conversions
__device__ __forceinline__ dfloat df_from_double(double v)
{
    uint32_t hb, lb;
    if (split_double_bits((uint64_t)__double_as_longlong(v), &hb, &lb)) {
        return {__uint_as_float(hb), __uint_as_float(lb)};
    }
    const float h = __double2float_rn(v);
    return {h, __double2float_rn(v - (double)h)};
}

__device__ __forceinline__ double df_to_double(dfloat x) { return (double)x.hi + (double)x.lo; }

}  // namespace iptgb
