// Compensated (Dot2) sums for the mixed form's precise contraction
// (mixed_point.cuh: second and higher derivatives of order >= 4 tables).
//
// A double-float value is an unevaluated sum hi + lo of two FP32 numbers. The
// compensated dot product Dot2 of Ogita, Rump and Oishi, "Accurate sum and
// dot product", SIAM J. Sci. Comput. 26(6), 2005, gives a result as accurate
// as if computed in twice the working precision: |error| <= u |x.y| +
// gamma_n^2 |x|.|y|, from FP32 instructions only. Its building blocks are
// Knuth's TwoSum and the FMA form of the exact product (TwoProd). Every
// rounding step is written with an explicit _rn intrinsic so that the
// compiler cannot contract or reassociate them.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace intp_gb300 {

struct DF {
    float hi, lo;
};

// s + e = a + b exactly (any a, b).
__device__ __forceinline__ DF df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return DF{s, e};
}

// Dot2 accumulator: the running sum is s + c (c collects the rounding errors
// of the products and of the sums of their high parts).
struct Dot2 {
    float s, c;
};

// acc += a * x for a double-float coefficient a = (a.x, a.y) and an operand
// x = xh + xl (xl = 0 when HAS_LO is false). The products a.y*xh and a.x*xl
// are below u of the leading product and enter the error term directly
// (their own rounding is of order u^2).
template <bool HAS_LO>
__device__ __forceinline__ void dot2_add(Dot2& acc, float2 a, float xh, float xl) {
    const float p = __fmul_rn(a.x, xh);
    float q = __fmaf_rn(a.x, xh, -p);
    q = __fmaf_rn(a.y, xh, q);
    if (HAS_LO) q = __fmaf_rn(a.x, xl, q);
    const DF t = df_two_sum(acc.s, p);
    acc.s = t.hi;
    acc.c = __fadd_rn(acc.c, __fadd_rn(t.lo, q));
}

// Normalised double-float value of an accumulator.
__device__ __forceinline__ DF dot2_value(const Dot2& acc) { return df_two_sum(acc.s, acc.c); }

}  // namespace intp_gb300
