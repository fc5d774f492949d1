// FP32 per-axis weights of the mixed-precision form: basis values of order
// O - k at the local offset u = x - t_c (Cox-de Boor, BSpline.hpp:83-111)
// followed by k transposed differencing steps (the derivative, BSpline.hpp:
// 489-520, moved from the control points onto the weights).
//
// Uniform axes away from clamped ends have knot differences that are exact
// multiples of dx, so the recursion runs on t = u / dx with compile-time
// constants and no table loads; elsewhere (clamped ends of non-periodic axes,
// non-uniform axes) it reads per-cell FP32 knot offsets and reciprocals.
#pragma once

#include "device_common.cuh"

namespace intp_gb300 {

// Right-aligned basis of spline order s <= O on unit-spaced knots at local
// coordinate t in [0, 1): knots at integer positions relative to the cell.
template <int O>
__device__ __forceinline__ void uniform_basis(float t, int s, float (&N)[O + 1]) {
#pragma unroll
    for (int k = 0; k < O; ++k) N[k] = 0.0f;
    N[O] = 1.0f;
#pragma unroll
    for (int i = 1; i <= O; ++i) {
        if (i <= s) {
            const int b = O - i;
            const float inv_i = 1.0f / static_cast<float>(i);
#pragma unroll
            for (int j = 0; j <= i; ++j) {
                // knots t_l = j - i, t_{r-1} = j, t_r = j + 1, t_{l+1} = j - i + 1
                float v = 0.0f;
                if (j > 0) v = N[b + j] * (t - static_cast<float>(j - i)) * inv_i;
                if (b + j < O) v += N[b + j + 1] * (static_cast<float>(j + 1) - t) * inv_i;
                N[b + j] = v;
            }
        }
    }
}

// Same recursion on tabulated knots: kd[j] = t_{c+j} - t_c (j = -O..O+1) and
// reciprocals rinv[a*O + s-1] = 1 / (t_{a+s} - t_a).
template <int O>
__device__ __forceinline__ void table_basis(const AxisDev& a, int64_t c, float u, int s, float (&N)[O + 1]) {
#pragma unroll
    for (int k = 0; k < O; ++k) N[k] = 0.0f;
    N[O] = 1.0f;
    if constexpr (O > 0) {
        const float* kd = a.kdf + c * (2 * O + 2) + O;
        float tk[2 * O];  // t_{c+o} - t_c for o = -O+1 .. O
#pragma unroll
        for (int m = 0; m < 2 * O; ++m) tk[m] = __ldg(kd - O + 1 + m);
#pragma unroll
        for (int i = 1; i <= O; ++i) {
            if (i <= s) {
                const int b = O - i;
#pragma unroll
                for (int j = 0; j <= i; ++j) {
                    float v = 0.0f;
                    if (j > 0)
                        v = N[b + j] * (u - tk[j - i + O - 1]) * __ldg(a.rinvf + (c - i + j) * O + (i - 1));
                    if (b + j < O)
                        v += N[b + j + 1] * (tk[j + O] - u) * __ldg(a.rinvf + (c - i + j + 1) * O + (i - 1));
                    N[b + j] = v;
                }
            }
        }
    }
}

// w <- M^T w for derivative order k with per-step factors alpha(m, kk).
template <int O, class Alpha>
__device__ __forceinline__ void transpose_difference(int k, float (&w)[O + 1], Alpha alpha) {
#pragma unroll
    for (int kk = 1; kk <= O; ++kk) {
        if (kk >= O - k + 1) {
            const int s0 = O - kk + 1;
#pragma unroll
            for (int i = 0; i <= O; ++i) {
                float v = (i >= s0) ? alpha(i, kk) * w[i] : w[i];
                if (i + 1 <= O && i + 1 >= s0) v -= alpha(i + 1, kk) * w[i + 1];
                w[i] = v;
            }
        }
    }
}

// Weights of derivative order k (0 <= k <= O) on axis `a` at span c, local
// offset u.
template <int O>
__device__ __forceinline__ void axis_weights32(const AxisDev& a, int64_t c, float u, int k, float (&w)[O + 1]) {
    if (a.uniform && c >= a.int_lo && c <= a.int_hi) {
        uniform_basis<O>(u * a.inv_dxf, O - k, w);
        const float id = a.inv_dxf;
        transpose_difference<O>(k, w, [id](int, int) { return id; });
    } else {
        table_basis<O>(a, c, u, O - k, w);
        const float* rv = a.rinvf;
        transpose_difference<O>(k, w, [rv, c](int m, int kk) {
            return static_cast<float>(kk) * __ldg(rv + (c + m - O) * O + (kk - 1));
        });
    }
}

}  // namespace intp_gb300
