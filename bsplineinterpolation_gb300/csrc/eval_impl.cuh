// Batched evaluation of value and derivatives (direct form: one thread per
// query point, control points gathered through L1/L2).
//
// Per point and axis: periodic wrap (BSpline.hpp:130-136), exact knot span
// (BSpline.hpp:125-157), Cox-de Boor basis (BSpline.hpp:83-111). Derivatives
// (BSpline.hpp:393-532) are applied to the basis instead of the control
// points: the reference differences the local control points k times,
//   Q_m <- k'(Q_m - Q_{m-1}) / (t_{c+m-O+k'} - t_{c+m-O}),
// which is a linear map M with result = N^T M P; the kernel forms
// w = M^T N once per axis (the transposed differencing) and contracts
// sum_i P_i prod_d w_d[i_d]. Both give the same value up to rounding.
//
// FP64 form: coordinates, basis and contraction in FP64 (parity form).
// Mixed form: span in exact integer arithmetic, local offset u = x - t_c from
// an exact split of x, basis and contraction in FP32 with FP32 control points.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "basis32.cuh"
#include "device_common.cuh"
#include "mixed_point.cuh"
#include "launch.hpp"

namespace intp_gb300 {

namespace eval_detail {

template <int O>
struct Basis64 {
    // Basis of spline order s (<= O) at x in span c, right-aligned.
    __device__ static void eval(const AxisDev& a, int64_t c, double x, int s, double (&N)[O + 1]) {
#pragma unroll
        for (int k = 0; k < O; ++k) N[k] = 0.0;
        N[O] = 1.0;
        if constexpr (O > 0) {
        // knots t[c-O+1 .. c+O]
        double tk[2 * O + 1];
#pragma unroll
        for (int m = 0; m < 2 * O; ++m) tk[m] = __ldg(a.knots + c - O + 1 + m);
#pragma unroll
        for (int i = 1; i <= O; ++i) {
            if (i <= s) {
                const int b = O - i;
#pragma unroll
                for (int j = 0; j <= i; ++j) {
                    // l = c - i + j, r = c + j + 1; tk index of t[c+o] is o + O - 1
                    double left = 0.0, right = 0.0;
                    if (j > 0) {
                        const int64_t l = c - i + j;
                        const double xl = x - tk[j - i + O - 1];
                        left = N[b + j] * xl * __ldg(a.rinv + l * O + (i - 1));
                    }
                    if (b + j < O) {
                        const int64_t l1 = c - i + j + 1;
                        const double xr = tk[j + 1 + O - 1] - x;
                        right = N[b + j + 1] * xr * __ldg(a.rinv + l1 * O + (i - 1));
                    }
                    N[b + j] = left + right;
                }
            }
        }
        }
    }
};

// w <- M^T w for derivative order k (basis of order O-k in w on entry).
template <int O, class R>
__device__ __forceinline__ void deriv_transform(const AxisDev& a, int64_t c, int k, R (&w)[O + 1]) {
    const R* rv;
    if constexpr (std::is_same<R, float>::value)
        rv = a.rinvf;
    else
        rv = a.rinv;
#pragma unroll
    for (int kk = 1; kk <= O; ++kk) {
        if (kk >= O - k + 1) {
            const int s0 = O - kk + 1;  // S = [s0, O]
            R alpha[O + 1];
#pragma unroll
            for (int m = 0; m <= O; ++m)
                alpha[m] = (m >= s0) ? static_cast<R>(kk) * __ldg(rv + (c + m - O) * O + (kk - 1))
                                     : static_cast<R>(1);
#pragma unroll
            for (int i = 0; i <= O; ++i) {
                R v = (i >= s0) ? alpha[i] * w[i] : w[i];
                if (i + 1 <= O && i + 1 >= s0) v -= alpha[i + 1] * w[i + 1];
                w[i] = v;
            }
        }
    }
}

__device__ __forceinline__ int64_t wrap_index(int64_t v, int64_t n, bool periodic) {
    if (!periodic) return v;
    v %= n;
    return v < 0 ? v + n : v;
}

constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

// Mixed-form outputs of one channel of one query (the per-query code of the
// binned kernel, so results are identical): operands relative to the query's
// central control point, with (LO) the control points' FP32 remainders
// added to their offsets from the bucket base cbase.
template <int D, int O, bool LO>
__device__ __forceinline__ void mixed_channel(const TableDev& t, const DerivPlan& plan, const int64_t (&cell)[D],
                                              const float (&xr)[D], const float (&base)[D][O + 1],
                                              const int64_t (&off)[D][O + 1], const float* __restrict__ cpc,
                                              const float* __restrict__ loc, void* __restrict__ out, int out_f32,
                                              int64_t o0, int C, int ch) {
    if (plan.precise) {
        // operands relative to the query's central control point, in
        // double-float (its FP32 value and remainder)
        int64_t oref = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) oref += off[d][ref_tap<O>()];
        const float rh = __ldg(cpc + oref), rl = LO ? __ldg(loc + oref) : 0.0f;
        precise_point_outputs<D, O>(
            t, plan, cell, xr, base, rh, rl,
            [&](const int (&ix)[D]) {
                int64_t o = 0;
#pragma unroll
                for (int d = 0; d < D; ++d) o += off[d][ix[d]];
                const float dh = __ldg(cpc + o) - rh;
                if constexpr (LO)
                    return dh + (__ldg(loc + o) - rl);
                else
                    return dh;
            },
            [out, out_f32, o0, C, ch](int k, float v) {
                const int64_t e = (o0 + k) * C + ch;
                if (out_f32)
                    static_cast<float*>(out)[e] = v;
                else
                    static_cast<double*>(out)[e] = static_cast<double>(v);
            });
        return;
    }
    const float cbase = LO ? __ldg(cpc + bucket_centre_offset<D, O>(t, cell)) : 0.0f;
    auto operand = [&](int64_t o) {
        const float h = __ldg(cpc + o);
        if constexpr (LO)
            return (h - cbase) + __ldg(loc + o);
        else
            return h;
    };
    int64_t oref = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) oref += off[d][ref_tap<O>()];
    const float cref = operand(oref);
    mixed_point_outputs<D, O>(
        t, plan, cell, xr, base, cref, cbase,
        [&](const int (&ix)[D]) {
            int64_t o = 0;
#pragma unroll
            for (int d = 0; d < D; ++d) o += off[d][ix[d]];
            return operand(o) - cref;
        },
        [out, out_f32, o0, C, ch](int k, float v) {
            const int64_t e = (o0 + k) * C + ch;
            if (out_f32)
                static_cast<float*>(out)[e] = v;
            else
                static_cast<double*>(out)[e] = static_cast<double>(v);
        });
}

// All outputs of one query point: xp holds its D coordinates, output k goes
// to out[o0 + k]. Shared by the direct kernel and the batched-table kernel.
// LO = false: a caller whose plan has no derivative output (the control
// points' remainders are never read) drops that contraction's code.
template <int D, int O, bool MIXED, bool LO = true>
__device__ __forceinline__ void eval_point(const TableDev& t, const double* __restrict__ xp, const DerivPlan& plan,
                                           void* __restrict__ out, int out_f32, int64_t o0) {
    using R = typename std::conditional<MIXED, float, double>::type;
    constexpr int W = O + 1;
    constexpr int ROWS = ipow(W, D - 1);
    const R* __restrict__ cp = static_cast<const R*>(t.ctrl);
    const int K = plan.k;
    int64_t cell[D];
    R xr[D];
    R base[D][W];
    int64_t off[D][W];
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const AxisDev& a = t.ax[d];
        double x = __ldg(xp + d);
        if (a.periodic) x = periodic_wrap(a, x);
        const int64_t h = a.uniform ? uniform_hint(a, x) : static_cast<int64_t>(O);
        const int64_t c = locate_span(a, O, knot_key(x), h);
        cell[d] = c;
        if constexpr (MIXED) {
            float xh, xl;
            split_double(x, xh, xl);
            const float u = (xh - __ldg(a.khi + c)) + (xl - __ldg(a.klo + c));
            xr[d] = u;
            axis_weights32<O>(a, c, u, 0, base[d]);
        } else {
            xr[d] = x;
            Basis64<O>::eval(a, c, x, O, base[d]);
        }
#pragma unroll
        for (int i = 0; i < W; ++i) off[d][i] = wrap_index(c - O + i, a.n, a.periodic) * a.stride;
    }
    // vector-valued tables: channel ch's control points start at
    // ch * chan_stride; the weights above are shared by all channels, and
    // output k of channel ch goes to out[(o0 + k) * C + ch]
    const int C = t.channels;
    if constexpr (MIXED) {
        for (int ch = 0; ch < C; ++ch) {
            const R* __restrict__ cpc = cp + ch * t.chan_stride;
            // the remainders matter for derivatives only (a value is within
            // FP32 rounding of the stored control points either way); 4D
            // tables contract the stored FP32 control points
            if constexpr (D <= 3 && LO) {
                if (t.ctrl_lo && plan.has_deriv) {
                    mixed_channel<D, O, true>(t, plan, cell, xr, base, off, cpc, t.ctrl_lo + ch * t.chan_stride, out,
                                              out_f32, o0, C, ch);
                    continue;
                }
            }
            mixed_channel<D, O, false>(t, plan, cell, xr, base, off, cpc, nullptr, out, out_f32, o0, C, ch);
        }
    } else {
        for (int k = 0; k < K; ++k) {
            R w[D][W];
            bool zero = false;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const int kd = plan.ord[k][d];
                if (kd > O) {
                    zero = true;
                } else if (kd == 0) {
#pragma unroll
                    for (int i = 0; i < W; ++i) w[d][i] = base[d][i];
                } else {
                    Basis64<O>::eval(t.ax[d], cell[d], xr[d], O - kd, w[d]);
                    deriv_transform<O, R>(t.ax[d], cell[d], kd, w[d]);
                }
            }
            for (int ch = 0; ch < C; ++ch) {
                const R* __restrict__ cpc = cp + ch * t.chan_stride;
                R acc = 0;
                if (!zero) {
                    if constexpr (ROWS <= 64) {
#pragma unroll
                        for (int r = 0; r < ROWS; ++r) {
                            int64_t o = 0;
                            R wr = 1;
                            int rem = r;
#pragma unroll
                            for (int d = D - 2; d >= 0; --d) {
                                const int i = rem % W;
                                rem /= W;
                                o += off[d][i];
                                wr *= w[d][i];
                            }
                            R s = 0;
#pragma unroll
                            for (int i = 0; i < W; ++i) s += w[D - 1][i] * __ldg(cpc + o + off[D - 1][i]);
                            acc += wr * s;
                        }
                    } else {
                        // large (O+1)^(D-1): runtime row loop, weights from local memory
#pragma unroll 1
                        for (int r = 0; r < ROWS; ++r) {
                            int64_t o = 0;
                            R wr = 1;
                            int rem = r;
                            for (int d = D - 2; d >= 0; --d) {
                                const int i = rem % W;
                                rem /= W;
                                o += off[d][i];
                                wr *= w[d][i];
                            }
                            R s = 0;
#pragma unroll
                            for (int i = 0; i < W; ++i) s += w[D - 1][i] * __ldg(cpc + o + off[D - 1][i]);
                            acc += wr * s;
                        }
                    }
                }
                const int64_t e = (o0 + k) * C + ch;
                if (out_f32)
                    static_cast<float*>(out)[e] = static_cast<float>(acc);
                else
                    static_cast<double*>(out)[e] = static_cast<double>(acc);
            }
        }
    }
}

template <int D, int O, bool MIXED>
__global__ void __launch_bounds__(128) eval_direct_kernel(TableDev t, const double* __restrict__ coords,
                                                          int64_t npts, DerivPlan plan,
                                                          void* __restrict__ out, int out_f32) {
    for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < npts;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x)
        eval_point<D, O, MIXED>(t, coords + p * D, plan, out, out_f32, p * plan.k);
}

}  // namespace eval_detail

}  // namespace intp_gb300
