// Double-word values (an unevaluated sum hi + lo of two FP32 numbers, about
// 48 significant bits) as the element type of the mixed form's line solves.
//
// The mixed form solves for control points in double-word arithmetic on the
// FP32 pipes: the band substitution (solve_line.cuh) runs unchanged with
// R = DW, each multiply-add c + a*b rounded to about 2^-47 relative, where the
// FP64 form rounds to 2^-53 at a fraction of the rate (GB300 issues FP64 at
// roughly 1/70 of FP32). The factor, the right-hand sides and the solution
// are double-words; the control points are stored as their two FP32 halves
// (ctrl + ctrl_lo).
//
// The building blocks are the classical error-free transformations: Knuth's
// TwoSum, Dekker's Fast2Sum and the FMA form of the exact product (TwoProd);
// the multiply-add and the product follow the double-word algorithms of
// Joldes, Muller and Popescu, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic", ACM TOMS 44(2), 2017, in their
// cheaper form (DWTimesDW with the low-order cross terms folded into one FMA
// chain, then a Fast2Sum renormalisation). Every rounding step is written
// with an explicit _rn intrinsic so that the compiler cannot contract or
// reassociate them.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace intp_gb300 {

struct alignas(8) DW {
    float hi, lo;
    DW() = default;
    __host__ __device__ constexpr DW(float h, float l) : hi(h), lo(l) {}
    // the substitution initialises its windows and sums with 0
    __host__ __device__ constexpr DW(int v) : hi(static_cast<float>(v)), lo(0.0f) {}
};

// s + e = a + b exactly (any a, b).
__device__ __forceinline__ DW dw_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return DW(s, e);
}

// s + e = a + b exactly when |a| >= |b| (or a = 0).
__device__ __forceinline__ DW dw_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return DW(s, __fsub_rn(b, __fsub_rn(s, a)));
}

// a * b: the exact product of the high parts plus the cross terms.
__device__ __forceinline__ DW dw_mul(DW a, DW b) {
    const float ph = __fmul_rn(a.hi, b.hi);
    float pl = __fmaf_rn(a.hi, b.hi, -ph);
    pl = __fmaf_rn(a.hi, b.lo, pl);
    pl = __fmaf_rn(a.lo, b.hi, pl);
    return dw_fast_two_sum(ph, pl);
}

// c + a * b.
__device__ __forceinline__ DW fma_r(DW a, DW b, DW c) {
    const float ph = __fmul_rn(a.hi, b.hi);
    float pl = __fmaf_rn(a.hi, b.hi, -ph);
    pl = __fmaf_rn(a.hi, b.lo, pl);
    pl = __fmaf_rn(a.lo, b.hi, pl);
    const DW s = dw_two_sum(c.hi, ph);
    const float t = __fadd_rn(__fadd_rn(c.lo, pl), s.lo);
    return dw_fast_two_sum(s.hi, t);
}

__device__ __forceinline__ DW operator-(DW a) { return DW(-a.hi, -a.lo); }

// a - b (the substitution uses it only to test finiteness: v - v == 0).
__device__ __forceinline__ DW operator-(DW a, DW b) {
    const DW s = dw_two_sum(a.hi, -b.hi);
    return dw_fast_two_sum(s.hi, __fadd_rn(s.lo, __fsub_rn(a.lo, b.lo)));
}

__device__ __forceinline__ DW& operator*=(DW& a, DW b) {
    a = dw_mul(a, b);
    return a;
}

__device__ __forceinline__ bool operator==(DW a, DW b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(DW a, DW b) { return !(a == b); }

// Host: the double-word nearest a double (hi the nearest float, lo the
// nearest float to the rest), zero halves always +0 (as the FP32 factor
// copies: decaying side-band entries that underflow would otherwise
// alternate in sign).
inline DW dw_from_double(double x) {
    float h = static_cast<float>(x);
    float l = static_cast<float>(x - static_cast<double>(h));
    if (h == 0.0f) h = 0.0f;
    if (l == 0.0f) l = 0.0f;
    return DW(h, l);
}

}  // namespace intp_gb300

// Read-only loads and warp shuffles of double-words, for the substitution
// code that is written for any element type (global scope, next to CUDA's
// own overloads).
__device__ __forceinline__ intp_gb300::DW __ldg(const intp_gb300::DW* p) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    return intp_gb300::DW(v.x, v.y);
}
__device__ __forceinline__ intp_gb300::DW __shfl_sync(unsigned mask, intp_gb300::DW v, int src, int width = 32) {
    return intp_gb300::DW(__shfl_sync(mask, v.hi, src, width), __shfl_sync(mask, v.lo, src, width));
}
__device__ __forceinline__ intp_gb300::DW __shfl_up_sync(unsigned mask, intp_gb300::DW v, unsigned d, int width = 32) {
    return intp_gb300::DW(__shfl_up_sync(mask, v.hi, d, width), __shfl_up_sync(mask, v.lo, d, width));
}
__device__ __forceinline__ intp_gb300::DW __shfl_down_sync(unsigned mask, intp_gb300::DW v, unsigned d,
                                                          int width = 32) {
    return intp_gb300::DW(__shfl_down_sync(mask, v.hi, d, width), __shfl_down_sync(mask, v.lo, d, width));
}
