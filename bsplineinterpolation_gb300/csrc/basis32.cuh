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

// Polynomial form of the uniform basis: on unit-spaced knots the O+1 basis
// functions of order O on a span are fixed polynomials in t = (x - t_c)/dx,
// and so are their derivatives. c[k][j][m] is the coefficient of t^m in
// d^k/dt^k of basis function j; it is built at compile time by running the
// Cox-de Boor recursion (BSpline.hpp:91-109) on polynomials.
template <int O>
struct UniformPoly {
    double c[O + 1][O + 1][O + 1];
};

template <int O>
constexpr UniformPoly<O> make_uniform_poly() {
    UniformPoly<O> r{};
    double N[O + 1][O + 1] = {};
    N[O][0] = 1.0;
    for (int i = 1; i <= O; ++i) {
        const int b = O - i;
        for (int j = 0; j <= i; ++j) {
            double v[O + 1] = {};
            if (j > 0)
                for (int m = 0; m < O; ++m) {
                    v[m + 1] += N[b + j][m] / i;
                    v[m] += N[b + j][m] * static_cast<double>(i - j) / i;
                }
            if (b + j < O)
                for (int m = 0; m < O; ++m) {
                    v[m] += N[b + j + 1][m] * static_cast<double>(j + 1) / i;
                    v[m + 1] -= N[b + j + 1][m] / i;
                }
            for (int m = 0; m <= O; ++m) N[b + j][m] = v[m];
        }
    }
    for (int k = 0; k <= O; ++k)
        for (int j = 0; j <= O; ++j)
            for (int m = 0; m + k <= O; ++m) {
                double f = 1.0;
                for (int q = m + 1; q <= m + k; ++q) f *= q;
                r.c[k][j][m] = N[j][m + k] * f;
            }
    return r;
}

// One coefficient as a compile-time scalar (folded into the instructions).
template <int O, int K, int J, int M>
struct UPolyCoef {
    static constexpr float value = static_cast<float>(make_uniform_poly<O>().c[K][J][M]);
};

// Horner evaluation of d^K B_J / dt^K at t (degree O - K).
template <int O, int K, int J, int M = 0>
__device__ __forceinline__ float uniform_poly_horner(float t) {
    if constexpr (M == O - K)
        return UPolyCoef<O, K, J, M>::value;
    else
        return fmaf(uniform_poly_horner<O, K, J, M + 1>(t), t, UPolyCoef<O, K, J, M>::value);
}

// Derivative-K weights on a uniform span: Horner in t, times dx^-K.
template <int O, int K, int J = 0>
__device__ __forceinline__ void uniform_poly_weights(float t, float scale, float (&w)[O + 1]) {
    if constexpr (J <= O) {
        w[J] = uniform_poly_horner<O, K, J>(t) * scale;
        uniform_poly_weights<O, K, J + 1>(t, scale, w);
    }
}

template <int O, int K = 0>
__device__ __forceinline__ void uniform_poly_dispatch(int k, float t, float inv_dx, float (&w)[O + 1]) {
    if constexpr (K <= O) {
        if (k == K) {
            float scale = 1.0f;
#pragma unroll
            for (int q = 0; q < K; ++q) scale *= inv_dx;
            uniform_poly_weights<O, K>(t, scale, w);
        } else {
            uniform_poly_dispatch<O, K + 1>(k, t, inv_dx, w);
        }
    }
}

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
        uniform_poly_dispatch<O>(k, u * a.inv_dxf, a.inv_dxf, w);
    } else {
        table_basis<O>(a, c, u, O - k, w);
        const float* rv = a.rinvf;
        transpose_difference<O>(k, w, [rv, c](int m, int kk) {
            return static_cast<float>(kk) * __ldg(rv + (c + m - O) * O + (kk - 1));
        });
    }
}

// Weights of the precise mixed path (mixed_point.cuh precise_point_outputs):
// value weights as axis_weights32; derivative weights on uniform interior
// spans from the Cox-de Boor recursion on unit knots (uniform_basis, a
// sequence of convex combinations) followed by the transposed differencing,
// instead of the monomial (Horner) form, whose coefficients grow and
// alternate in sign with the degree: at order 7 the Horner second-derivative
// weights carry errors of several FP32 ulps of the largest weight. On
// uniform knots every differencing factor k' / (t_{a+k'} - t_a) is 1/dx.
template <int O>
__device__ __forceinline__ void axis_weights32_precise(const AxisDev& a, int64_t c, float u, int k,
                                                       float (&w)[O + 1]) {
    if (k == 0 || !(a.uniform && c >= a.int_lo && c <= a.int_hi)) {
        axis_weights32<O>(a, c, u, k, w);
        return;
    }
    uniform_basis<O>(u * a.inv_dxf, O - k, w);
    const float inv = a.inv_dxf;
    transpose_difference<O>(k, w, [inv](int, int) { return inv; });
}

}  // namespace intp_gb300
