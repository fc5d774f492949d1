// Device-side shared definitions: table descriptor, exact knot-span location,
// and the integer double->float split used by the mixed-precision path.
//
// GB300 executes FP64 (and f64<->f32 conversions) at roughly 1/70 of its FP32
// rate, so the mixed path keeps every per-point FP64 instruction off the
// critical path: knot spans are found by exact comparisons of order-preserving
// int64 keys, and local offsets are formed from an exact (hi, lo) split of
// the coordinate computed with integer operations.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace intp_gb300 {

constexpr int kDevMaxDim = 4;
constexpr int kDevMaxOrder = 7;
constexpr int kMaxDeriv = 16;

struct AxisDev {
    int64_t n;        // control points along the axis
    int64_t nknots;
    int64_t stride;   // control-point stride (elements)
    int32_t periodic;
    int32_t uniform;
    double lo, hi, period;   // BSpline::range_ and hi - lo
    float hint_x0;           // uniform axes: knots[i] ~ hint_x0 + (i - hint_off) / hint_inv_dx
    float hint_inv_dx;
    float hint_off;
    float inv_dxf;           // uniform axes: 1 / dx in FP32
    int64_t int_lo, int_hi;  // spans whose basis knots are all uniformly spaced
    int64_t ncells;          // spans an evaluation can land in: [O, O + ncells)
    const double* knots;     // [nknots]
    const long long* keys;   // [nknots] order-preserving keys of the knots
    const double* rinv;      // [nknots * O]  1 / (t[a+s] - t[a]), s = 1..O (0 if equal)
    const float* rinvf;      // FP32 copy of rinv
    const float* kdf;        // [nknots * (2O+2)]  t[a+j] - t[a], j = -O..O+1 (FP32)
    const float* khi;        // [nknots] high FP32 part of the knot (truncated)
    const float* klo;        // [nknots] remainder t - khi rounded to FP32
};

struct TableDev {
    int32_t dim;
    int32_t order;
    AxisDev ax[kDevMaxDim];
    const void* ctrl;        // float (mixed) or double (fp64) control points, row-major
    // mixed form after refinement: the FP32 remainder of every control point
    // (control point = ctrl + ctrl_lo as a double-float), else NULL
    const float* ctrl_lo;
    int32_t channels;        // values per mesh point (vector-valued tables; 1 = scalar)
    int64_t chan_stride;     // control points of one channel (channel-major storage)
};

// Spatial buckets of the binned evaluation. Local span index l_d = c_d - O
// of a query; bucket coordinate l_d >> lb[d] (B_d = 2^lb[d] spans per bucket
// and axis); tile of control points P_d = B_d + O per axis, row-major with
// strides tstride[d].
struct BinGeom {
    int32_t dim;
    int32_t lb[kDevMaxDim];
    int32_t nb[kDevMaxDim];
    int32_t P[kDevMaxDim];
    int32_t shift[kDevMaxDim];   // bit offset of l_d & (B_d - 1) in the packed span (row-major: last axis lowest)
    int32_t tstride[kDevMaxDim];
    int64_t nbuckets;
    int32_t tile_elems;
    int32_t smem_buckets;        // bucket count, or 0 when too many: the table evaluates directly
};

// Derivative orders of up to kMaxDeriv outputs per point. Outputs with the
// same orders on axes 1..D-1 form a group: they share the contraction over
// those axes and differ only in their axis-0 weights.
struct DerivPlan {
    int32_t k;                      // number of outputs
    int8_t ord[kMaxDeriv][kDevMaxDim];
    int32_t ngroups;
    int8_t group_rep[kMaxDeriv];    // an output of each group
    int8_t out_group[kMaxDeriv];    // group of each output
    int32_t simple;                 // one group, all orders on axes 1..D-1 zero
    int32_t has_deriv;              // some output has a derivative order above 0
    // mixed form: a derivative of order >= 2 on a table of order >= 4, which
    // takes the precise per-query contraction (mixed_point.cuh)
    int32_t precise;
};

// Spans per bucket (log2, per axis) of the binned evaluation, fixed per
// dimension so the shared-memory tile has compile-time strides.
__host__ __device__ constexpr int bucket_log2(int dim, int axis) {
    return dim == 1 ? 12 : dim == 2 ? 6 : 4;
}

// Division of 32-bit unsigned integers below 2^31 by a fixed divisor d >= 1
// as a multiply-high, add and shift (Granlund and Montgomery, "Division by
// invariant integers using multiplication", PLDI 1994, round-up variant):
// l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, n / d = (mulhi(m, n)
// + n) >> l.
struct FastDiv {
    uint32_t d, m;
    int l;
    __host__ __device__ static FastDiv make(uint32_t d) {
        FastDiv f{};
        f.d = d;
        f.l = 0;
        while ((uint64_t{1} << f.l) < d) ++f.l;
        f.m = static_cast<uint32_t>(((uint64_t{1} << 32) * ((uint64_t{1} << f.l) - d)) / d + 1);
        return f;
    }
    __device__ __forceinline__ uint32_t div(uint32_t n) const { return (__umulhi(m, n) + n) >> l; }
};

// Order-preserving integer key of a double: a < b  <=>  key(a) < key(b) for
// all non-NaN values, with -0 mapped onto +0 (IEEE compares them equal).
__host__ __device__ __forceinline__ long long knot_key_bits(unsigned long long b) {
    if (b == 0x8000000000000000ULL) b = 0;
    const long long s = static_cast<long long>(b);
    return s ^ ((s >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}

__device__ __forceinline__ long long knot_key(double x) {
    return knot_key_bits(static_cast<unsigned long long>(__double_as_longlong(x)));
}

// High part of x as a float: sign, exponent and the top 23 mantissa bits of the
// double (truncation). Tiny magnitudes map to 0, huge ones to infinity.
__host__ __device__ __forceinline__ uint32_t split_hi_bits(unsigned long long b) {
    const uint32_t hi = static_cast<uint32_t>(b >> 32);
    const uint32_t sign = hi & 0x80000000u;
    const int e = static_cast<int>((hi >> 20) & 0x7FFu);
    const int ef = e - 1023 + 127;
    if (ef <= 0) return sign;
    if (ef >= 255) return sign | 0x7F800000u;
    const uint32_t mant = ((hi & 0xFFFFFu) << 3) | (static_cast<uint32_t>(b >> 29) & 7u);
    return sign | (static_cast<uint32_t>(ef) << 23) | mant;
}

// Exact split x = hi + lo (lo rounded to FP32) without FP64 instructions.
__device__ __forceinline__ void split_double(double x, float& hi, float& lo) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    const uint32_t hb = split_hi_bits(b);
    hi = __int_as_float(static_cast<int>(hb));
    const uint32_t top = static_cast<uint32_t>(b >> 32);
    const int e = static_cast<int>((top >> 20) & 0x7FFu);
    const int ef = e - 1023 + 127;
    // remainder: low 29 mantissa bits of the double (their top 23 kept), worth
    // rem * 2^(e - 1075); only meaningful when hi is a normal float
    const uint32_t rem = (static_cast<uint32_t>(b) & 0x1FFFFFFFu) >> 6;
    const int se = e - 1069 + 127;  // exponent field of 2^(e - 1075 + 6)
    float scale = 0.0f;
    if (ef > 0 && ef < 255 && se > 0) scale = __int_as_float(se << 23);
    // rem < 2^23: exact conversion through the 2^23 magic constant
    const float remf = __int_as_float(static_cast<int>(0x4B000000u | rem)) - 8388608.0f;
    const float mag = remf * scale;
    lo = (top & 0x80000000u) ? -mag : mag;
}

// Approximate float value of a double, from integer operations only.
__device__ __forceinline__ float double_to_float_trunc(double x) {
    return __int_as_float(static_cast<int>(split_hi_bits(
        static_cast<unsigned long long>(__double_as_longlong(x)))));
}

// Periodic wrap of BSpline::get_knot_iter (BSpline.hpp:130-136), in FP64 with
// the reference's exact operation order. Returns the wrapped coordinate.
__device__ __forceinline__ double periodic_wrap(const AxisDev& a, double x) {
    const double r = __dadd_rn(__dadd_rn(a.lo, fmod(__dsub_rn(x, a.lo), a.period)),
                               (x < a.lo ? a.period : 0.0));
    return r;
}

// Knot span of BSpline::get_knot_iter (BSpline.hpp:125-157): the largest
// j in [O+1, last] with t[j] <= x, or O if there is none, where
// last = nknots - O - 2. Comparisons use exact integer keys. `hint` is any
// guess; it is verified before it is used.
__device__ __forceinline__ int64_t locate_span(const AxisDev& a, int order, long long kx,
                                               int64_t hint) {
    const int64_t lastc = a.nknots - order - 2;
    int64_t h = hint < order ? order : (hint > lastc ? lastc : hint);
    // accept h when t[h] <= x < t[h+1], or at the clamped ends
    const long long k0 = __ldg(a.keys + h), k1 = __ldg(a.keys + h + 1);
    const bool lo_ok = (h == order) || (k0 <= kx);
    const bool hi_ok = (h == lastc) || (kx < k1);
    if (lo_ok && hi_ok) return h;
    // one step either way covers an off-by-one hint
    if (!hi_ok && h + 1 <= lastc) {
        const long long k2 = (h + 1 == lastc) ? 0 : __ldg(a.keys + h + 2);
        if (h + 1 == lastc || kx < k2) return h + 1;
    }
    if (!lo_ok && h - 1 >= order) {
        const long long km = __ldg(a.keys + h - 1);
        if (h - 1 == order || km <= kx) return h - 1;
    }
    // binary search: count of knots in [O+1, last] that are <= x
    int64_t lo = order + 1, hi = lastc + 1;  // search [lo, hi)
    while (lo < hi) {
        const int64_t mid = lo + ((hi - lo) >> 1);
        if (__ldg(a.keys + mid) <= kx)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo - 1;
}

// locate_span with 32-bit indices (axes of fewer than 2^31 knots): the same
// verified-hint search, so the same span.
__device__ __forceinline__ int locate_span32(const AxisDev& a, int order, long long kx, int hint) {
    const int lastc = static_cast<int>(a.nknots) - order - 2;
    const int h = hint < order ? order : (hint > lastc ? lastc : hint);
    const long long k0 = __ldg(a.keys + h), k1 = __ldg(a.keys + h + 1);
    const bool lo_ok = (h == order) || (k0 <= kx);
    const bool hi_ok = (h == lastc) || (kx < k1);
    if (lo_ok && hi_ok) return h;
    if (!hi_ok && h + 1 <= lastc) {
        if (h + 1 == lastc || kx < __ldg(a.keys + h + 2)) return h + 1;
    }
    if (!lo_ok && h - 1 >= order) {
        if (h - 1 == order || __ldg(a.keys + h - 1) <= kx) return h - 1;
    }
    int lo = order + 1, hi = lastc + 1;
    while (lo < hi) {
        const int mid = lo + ((hi - lo) >> 1);
        if (__ldg(a.keys + mid) <= kx)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo - 1;
}

// uniform_hint as a 32-bit index, clamped to [-1, nknots].
__device__ __forceinline__ int uniform_hint32(const AxisDev& a, float xf) {
    float v = floorf((xf - a.hint_x0) * a.hint_inv_dx + a.hint_off);
    if (!(v > -1.0f)) v = -1.0f;  // also NaN
    const float top = static_cast<float>(a.nknots);
    if (v > top) v = top;
    return static_cast<int>(v);
}

// FP32 hint of the span on a uniform axis (integer-derived float of x).
__device__ __forceinline__ int64_t uniform_hint(const AxisDev& a, double x) {
    const float xf = double_to_float_trunc(x);
    const float v = floorf((xf - a.hint_x0) * a.hint_inv_dx + a.hint_off);
    if (!(v > -1.0e18f) || !(v < 1.0e18f)) return v > 0.0f ? a.nknots : 0;
    return static_cast<int64_t>(v);
}

}  // namespace intp_gb300
