// Outputs of one query in the mixed form, shared by the direct and the
// binned evaluation kernels so both produce identical results.
//
// Operands. A control point enters as v = ctrl where the table keeps FP32
// control points only, and as v = (ctrl - cbase) + ctrl_lo where the refined
// solve kept each point's FP32 remainder; cbase is the control point at the
// centre of the query's bucket tile (the binned kernel forms v once per tile
// element when it stages the tile). The contraction then reads v relative to
// the query's own central tap, cref = v at index ref_tap<O>() on every axis:
// value weights sum to 1 and derivative weights to 0, so the FP32 rounding of
// the weights and of the partial sums scales with the variation across the
// query's stencil only. The value adds cref and cbase back.
//
// Both matter for derivatives: FP32 storage alone rounds each control point
// by up to 2^-24 of its magnitude, and a reference shared by a whole tile
// leaves operands as large as half a tile's variation; a first derivative
// multiplies either by about 1/dx (above 1e-6 relative on a 256-point axis).
//
// Outputs sharing their derivative orders on axes 1..D-1 form a group and
// share the contraction over those axes; each then applies its own axis-0
// weights.
#pragma once

#include "basis32.cuh"
#include "device_common.cuh"
#include "dot2.cuh"

namespace intp_gb300 {

constexpr int ipow_i(int b, int e) { return e == 0 ? 1 : b * ipow_i(b, e - 1); }

// Stencil position (on every axis) of the reference control point: the tap
// nearest the query's position within its O + 1 taps.
template <int O>
constexpr int ref_tap() {
    return (O + 1) / 2;
}

// fetch(idx) returns the operand of control point (c_d - O + idx_d)_d minus
// cref; emit(k, v) stores output k.
template <int D, int O, class Fetch, class Emit>
__device__ __forceinline__ void mixed_point_outputs(const TableDev& t, const DerivPlan& plan, const int64_t (&c)[D],
                                                    const float (&u)[D], const float (&base)[D][O + 1], float cref,
                                                    float cbase, const Fetch& fetch, const Emit& emit) {
    constexpr int W = O + 1;
    constexpr int ROWS1 = D >= 2 ? ipow_i(W, D - 2) : 1;  // rows over axes 1..D-2
    const int K = plan.k;
    for (int grp = 0; grp < plan.ngroups; ++grp) {
        const int rep = plan.group_rep[grp];
        float w[D][W];
        bool zero = false;
#pragma unroll
        for (int d = 1; d < D; ++d) {
            const int kd = plan.ord[rep][d];
            if (kd > O) {
                zero = true;
            } else if (kd == 0) {
#pragma unroll
                for (int i = 0; i < W; ++i) w[d][i] = base[d][i];
            } else {
                axis_weights32<O>(t.ax[d], c[d], u[d], kd, w[d]);
            }
        }
        float Pz[W];
        // a stencil above 1024 operands (4D at orders 6 and 7) keeps the
        // axis-0 loop rolled: the same operations in the same order, with
        // compile time bounded
        constexpr int kUnrollI0 = W * ROWS1 * W <= 1024 ? W : 1;
#pragma unroll kUnrollI0
        for (int i0 = 0; i0 < W; ++i0) {
            float acc = 0.0f;
#pragma unroll
            for (int rw = 0; rw < ROWS1; ++rw) {
                int idx[D];
                idx[0] = i0;
                float wr = 1.0f;
                int rem = rw;
#pragma unroll
                for (int d = D - 2; d >= 1; --d) {
                    idx[d] = rem % W;
                    rem /= W;
                    wr *= w[d][idx[d]];
                }
                if constexpr (D == 1) {
                    acc = fetch(idx);
                } else {
                    float s = 0.0f;
#pragma unroll
                    for (int i = 0; i < W; ++i) {
                        idx[D - 1] = i;
                        s += w[D - 1][i] * fetch(idx);
                    }
                    acc += wr * s;
                }
            }
            Pz[i0] = acc;
        }
        for (int k = 0; k < K; ++k) {
            if (plan.out_group[k] != grp) continue;
            const int k0 = plan.ord[k][0];
            float v = 0.0f;
            if (!zero && k0 <= O) {
                float wl[W];
                if (k0 == 0) {
#pragma unroll
                    for (int i = 0; i < W; ++i) wl[i] = base[0][i];
                } else {
                    axis_weights32<O>(t.ax[0], c[0], u[0], k0, wl);
                }
#pragma unroll
                for (int i = 0; i < W; ++i) v += wl[i] * Pz[i];
                bool value_out = k0 == 0;
#pragma unroll
                for (int d = 1; d < D; ++d) value_out = value_out && plan.ord[k][d] == 0;
                if (value_out) v = (v + cref) + cbase;
            }
            emit(k, v);
        }
    }
}

// Outputs of one query in the precise mixed form (DerivPlan::precise: a
// derivative of order >= 2 on a table of order >= 4). Three changes from
// mixed_point_outputs, each needed to hold such outputs within 1e-6 of
// their scale (an FP32 emulation of the periodic order-7 workload put the
// plain form's second derivatives at 2e-6 and this form's at 6e-7):
//  - operands relative to the query's own central control point in
//    double-float, (c_hi - ref_hi) + (c_lo - ref_lo), so their rounding
//    scales with the variation across the stencil, not across a tile;
//  - derivative weights from the basis recursion (axis_weights32_precise);
//  - compensated accumulation (Dot2, dot2.cuh) of every partial sum
//    of the separable contraction, carried as double-floats between axes.
// fetch(idx) returns the FP32 operand of control point (c_d - O + idx_d)_d;
// ref = ref_hi + ref_lo is the central control point, added back to values.
template <int D, int O, class Fetch, class Emit>
__device__ __forceinline__ void precise_point_outputs(const TableDev& t, const DerivPlan& plan,
                                                      const int64_t (&c)[D], const float (&u)[D],
                                                      const float (&base)[D][O + 1], float ref_hi, float ref_lo,
                                                      const Fetch& fetch, const Emit& emit) {
    constexpr int W = O + 1;
    constexpr int ROWS1 = D >= 2 ? ipow_i(W, D - 2) : 1;  // rows over axes 1..D-2
    const int K = plan.k;
    for (int grp = 0; grp < plan.ngroups; ++grp) {
        const int rep = plan.group_rep[grp];
        float w[D][W];
        bool zero = false;
#pragma unroll
        for (int d = 1; d < D; ++d) {
            const int kd = plan.ord[rep][d];
            if (kd > O) {
                zero = true;
            } else if (kd == 0) {
#pragma unroll
                for (int i = 0; i < W; ++i) w[d][i] = base[d][i];
            } else {
                axis_weights32_precise<O>(t.ax[d], c[d], u[d], kd, w[d]);
            }
        }
        float Ph[W], Pl[W];
        constexpr int kUnrollI0 = W * ROWS1 * W <= 1024 ? W : 1;
#pragma unroll kUnrollI0
        for (int i0 = 0; i0 < W; ++i0) {
            Dot2 acc{0.0f, 0.0f};
#pragma unroll
            for (int rw = 0; rw < ROWS1; ++rw) {
                int idx[D];
                idx[0] = i0;
                float wr = 1.0f;
                int rem = rw;
#pragma unroll
                for (int d = D - 2; d >= 1; --d) {
                    idx[d] = rem % W;
                    rem /= W;
                    wr *= w[d][idx[d]];
                }
                if constexpr (D == 1) {
                    acc.s = fetch(idx);
                } else {
                    Dot2 row{0.0f, 0.0f};
#pragma unroll
                    for (int i = 0; i < W; ++i) {
                        idx[D - 1] = i;
                        dot2_add<false>(row, make_float2(w[D - 1][i], 0.0f), fetch(idx), 0.0f);
                    }
                    const DF rv = dot2_value(row);
                    if constexpr (D == 2) {
                        acc = Dot2{rv.hi, rv.lo};
                    } else {
                        dot2_add<true>(acc, make_float2(wr, 0.0f), rv.hi, rv.lo);
                    }
                }
            }
            const DF pv = dot2_value(acc);
            Ph[i0] = pv.hi;
            Pl[i0] = pv.lo;
        }
        for (int k = 0; k < K; ++k) {
            if (plan.out_group[k] != grp) continue;
            const int k0 = plan.ord[k][0];
            float v = 0.0f;
            if (!zero && k0 <= O) {
                float wl[W];
                if (k0 == 0) {
#pragma unroll
                    for (int i = 0; i < W; ++i) wl[i] = base[0][i];
                } else {
                    axis_weights32_precise<O>(t.ax[0], c[0], u[0], k0, wl);
                }
                Dot2 fin{0.0f, 0.0f};
#pragma unroll
                for (int i = 0; i < W; ++i) dot2_add<true>(fin, make_float2(wl[i], 0.0f), Ph[i], Pl[i]);
                v = __fadd_rn(fin.s, fin.c);
                bool value_out = k0 == 0;
#pragma unroll
                for (int d = 1; d < D; ++d) value_out = value_out && plan.ord[k][d] == 0;
                if (value_out) v = ref_hi + (v + ref_lo);
            }
            emit(k, v);
        }
    }
}

// Index of the control point at the centre of the bucket tile holding span
// c (the operands' base cbase), for each axis.
template <int D, int O>
__device__ __forceinline__ int64_t bucket_centre_offset(const TableDev& t, const int64_t (&c)[D]) {
    int64_t off = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const AxisDev& a = t.ax[d];
        const int lb = bucket_log2(D, d);
        const int64_t org = ((c[d] - O) >> lb) << lb;
        int64_t gi = org + ((1 << lb) + O) / 2;
        gi = a.periodic ? gi % a.n : (gi < a.n ? gi : a.n - 1);
        off += gi * a.stride;
    }
    return off;
}

}  // namespace intp_gb300
