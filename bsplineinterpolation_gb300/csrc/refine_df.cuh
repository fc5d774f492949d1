// Double-float arithmetic of the mixed form's iterative refinement, shared by
// the single-table build (solve_kernels.cu) and the batched build (batch.cu)
// so both round identically.
//
// A double-float value is an unevaluated sum hi + lo of two FP32 numbers with
// |lo| <= ulp(hi) / 2: about 48 significant bits from FP32 arithmetic only.
// GB300's FP32 pipes are many times faster than its FP64 ones, so the
// refinement residual r = F - A c (the one step that needs more than FP32)
// runs in double-float instead of FP64, and refined control points are kept
// as double-floats (ctrl + ctrl_lo): FP32 storage alone rounds every control
// point by up to 2^-24 of its magnitude, and a first derivative multiplies
// that by about 1/dx -- above 1e-6 of the derivative on a 256-point axis.
//
// The building blocks are the classical error-free transformations (Knuth's
// TwoSum, Dekker's Fast2Sum, the FMA form of TwoProd), the compensated dot
// product Dot2 of Ogita, Rump and Oishi, "Accurate sum and dot product",
// SIAM J. Sci. Comput. 26(6), 2005 (the result is as accurate as if computed
// in twice the working precision: |error| <= u |x.y| + gamma_n^2 |x|.|y|),
// and the double-word addition of Joldes, Muller and Popescu, "Tight and
// rigorous error bounds for basic building blocks of double-word
// arithmetic", ACM TOMS 44(2), 2017 (DWPlusFP, relative error below 2u^2,
// u = 2^-24). The residual needs only an absolute error well below the
// residual itself (about kappa * u * |F|), which Dot2 gives with a quarter
// of the operations of full double-word products and sums. Every rounding
// step is written with an explicit _rn intrinsic so that the compiler cannot
// contract or reassociate them.
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

// s + e = a + b exactly when |a| >= |b| (or a = 0).
__device__ __forceinline__ DF df_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return DF{s, e};
}

// x + y, y a single float (DWPlusFP).
__device__ __forceinline__ DF df_add_f(DF x, float y) {
    const DF s = df_two_sum(x.hi, y);
    const float v = __fadd_rn(x.lo, s.lo);
    return df_fast_two_sum(s.hi, v);
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

// One element of a residual pass along one axis, element-parallel form:
// acc += sign * (row i of the axis' collocation matrix) times the line whose
// element k sits at hi[base + k * S] (+ lo[...] when HAS_LO). The row is a
// band of 2*band+1 double-float values (tap d: column i - band + d, cyclic
// on a periodic axis); zero taps are skipped, the others summed in tap
// order.
template <bool HAS_LO, class I>
__device__ __forceinline__ void dot2_band_row(Dot2& acc, float sign, const float* __restrict__ hi,
                                              const float* __restrict__ lo, I base, int i, int n, I S, int band,
                                              bool periodic, const float2* __restrict__ val) {
    const int W = 2 * band + 1;
    for (int d = 0; d < W; ++d) {
        float2 a = __ldg(val + i * W + d);
        if (a.x == 0.0f && a.y == 0.0f) continue;
        a.x *= sign;
        a.y *= sign;
        int c = i - band + d;
        if (periodic) c = c < 0 ? c + n : (c >= n ? c - n : c);
        const I j = base + static_cast<I>(c) * S;
        dot2_add<HAS_LO>(acc, a, __ldg(hi + j), HAS_LO ? __ldg(lo + j) : 0.0f);
    }
}

// dot2_band_row with the band, the periodicity and the sign (NEG: -1) known
// at compile time: taps unrolled, the negation folded into the products,
// the same values in the same order. (A zero high part implies a zero low
// part: the low part is the rounding of the coefficient minus its high
// part.)
template <int BAND, bool PERIODIC, bool HAS_LO, bool NEG, class I>
__device__ __forceinline__ void dot2_band_row_t(Dot2& acc, const float* __restrict__ hi, const float* __restrict__ lo,
                                                I base, int i, int n, I S, const float2* __restrict__ val) {
    constexpr int W = 2 * BAND + 1;
    const float2* __restrict__ row = val + i * W;
#pragma unroll
    for (int d = 0; d < W; ++d) {
        float2 a = __ldg(row + d);
        if (a.x == 0.0f) continue;
        if (NEG) {
            a.x = -a.x;
            a.y = -a.y;
        }
        int c = i - BAND + d;
        if (PERIODIC) c = c < 0 ? c + n : (c >= n ? c - n : c);
        const I j = base + static_cast<I>(c) * S;
        dot2_add<HAS_LO>(acc, a, __ldg(hi + j), HAS_LO ? __ldg(lo + j) : 0.0f);
    }
}

// ---- two independent accumulations per instruction ----
// Blackwell's packed FP32x2 add / multiply / FMA carry out the same IEEE
// single-precision operation, rounded to nearest, on each half of a register
// pair, so the x2 forms below give, lane by lane, exactly the results of the
// scalar forms above (a - b is fma(b, -1, a), one rounding of the exact
// difference, as __fsub_rn). Two elements of a residual pass then cost the
// instructions of one.
struct Dot2x2 {
    float2 s, c;
};

__device__ __forceinline__ float2 sub2_rn(float2 a, float2 b) {
    return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}

// s + e = a + b exactly, per lane (df_two_sum).
__device__ __forceinline__ void df_two_sum2(float2 a, float2 b, float2& s, float2& e) {
    s = __fadd2_rn(a, b);
    const float2 bb = sub2_rn(s, a);
    e = __fadd2_rn(sub2_rn(a, sub2_rn(s, bb)), sub2_rn(b, bb));
}

// dot2_add per lane: acc += (ahi + alo) * (xh + xl).
template <bool HAS_LO>
__device__ __forceinline__ void dot2_add2(Dot2x2& acc, float2 ahi, float2 alo, float2 xh, float2 xl) {
    const float2 p = __fmul2_rn(ahi, xh);
    float2 q = __ffma2_rn(ahi, xh, make_float2(-p.x, -p.y));
    q = __ffma2_rn(alo, xh, q);
    if (HAS_LO) q = __ffma2_rn(ahi, xl, q);
    float2 t;
    df_two_sum2(acc.s, p, acc.s, t);
    acc.c = __fadd2_rn(acc.c, __fadd2_rn(t, q));
}

// Normalised double-float value of an accumulator.
__device__ __forceinline__ DF dot2_value(const Dot2& acc) { return df_two_sum(acc.s, acc.c); }

// Refined control point: (c + lo) + corr as a double-float; lo is taken as
// zero on the first step (has_lo false).
__device__ __forceinline__ void df_correct(float& c, float& lo, float corr, bool has_lo) {
    const DF r = df_add_f(DF{c, has_lo ? lo : 0.0f}, corr);
    c = r.hi;
    lo = r.lo;
}

}  // namespace intp_gb300
