// Evaluation proxies: the knot spans and basis weights of a set of points,
// computed once, then used to evaluate any number of tables that share the
// knots (InterpolationFunctionTemplate::eval_proxy, InterpolationTemplate.hpp:
// 145-176; InterpolationFunction::eval_proxy, Interpolation.hpp:493-503;
// BSpline::pre_calc_coef, BSpline.hpp:250-296).
//
// The reference precomputes one point's basis for reuse across functions
// built from one template. Here a proxy holds npts points: per point and
// axis its span, its offset (FP64 coordinate in the FP64 form, FP32 local
// offset in the mixed form) and its O+1 value weights, in device memory. One
// launch then evaluates a list of tables at every point (a thread per point,
// the tables in turn), so the locate and basis work is paid once for all of
// them. Each table's value is computed with the direct kernel's arithmetic
// (eval_impl.cuh eval_point), so it equals what intp_eval returns for the
// same table and points on the direct path.
#include <type_traits>

#include "eval_impl.cuh"

namespace intp_gb300 {

namespace {

using eval_detail::Basis64;
using eval_detail::ipow;
using eval_detail::wrap_index;

template <int D, int O, bool MIXED>
__global__ void __launch_bounds__(256) proxy_build_kernel(TableDev t, const double* __restrict__ coords, int64_t npts,
                                                          int64_t* __restrict__ cells, void* __restrict__ xr_out,
                                                          void* __restrict__ base_out) {
    using R = typename std::conditional<MIXED, float, double>::type;
    constexpr int W = O + 1;
    R* xr = static_cast<R*>(xr_out);
    R* base = static_cast<R*>(base_out);
    for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; q < npts;
         q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const AxisDev& a = t.ax[d];
            double x = __ldg(coords + q * D + d);
            if (a.periodic) x = periodic_wrap(a, x);
            const int64_t h = a.uniform ? uniform_hint(a, x) : static_cast<int64_t>(O);
            const int64_t c = locate_span(a, O, knot_key(x), h);
            R w[W];
            if constexpr (MIXED) {
                float xh, xl;
                split_double(x, xh, xl);
                const float u = (xh - __ldg(a.khi + c)) + (xl - __ldg(a.klo + c));
                xr[q * D + d] = u;
                axis_weights32<O>(a, c, u, 0, w);
            } else {
                xr[q * D + d] = x;
                Basis64<O>::eval(a, c, x, O, w);
            }
            cells[q * D + d] = c;
#pragma unroll
            for (int i = 0; i < W; ++i) base[(q * D + d) * W + i] = w[i];
        }
    }
}

template <int D, int O, bool MIXED>
__global__ void __launch_bounds__(256) proxy_eval_kernel(const TableDev* __restrict__ tables, int ntables,
                                                         int64_t npts, const int64_t* __restrict__ cells,
                                                         const void* __restrict__ xr_in,
                                                         const void* __restrict__ base_in, DerivPlan plan,
                                                         void* __restrict__ out, int out_f32) {
    using R = typename std::conditional<MIXED, float, double>::type;
    constexpr int W = O + 1;
    constexpr int ROWS = ipow(W, D - 1);
    const R* xrp = static_cast<const R*>(xr_in);
    const R* bp = static_cast<const R*>(base_in);
    for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; q < npts;
         q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t cell[D];
        R xr[D];
        R base[D][W];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            cell[d] = __ldg(cells + q * D + d);
            xr[d] = __ldg(xrp + q * D + d);
#pragma unroll
            for (int i = 0; i < W; ++i) base[d][i] = __ldg(bp + (q * D + d) * W + i);
        }
        for (int j = 0; j < ntables; ++j) {
            const TableDev& t = tables[j];
            int64_t off[D][W];
#pragma unroll
            for (int d = 0; d < D; ++d)
#pragma unroll
                for (int i = 0; i < W; ++i)
                    off[d][i] = wrap_index(cell[d] - O + i, t.ax[d].n, t.ax[d].periodic) * t.ax[d].stride;
            const int64_t o0 = q * ntables + j;
            if constexpr (MIXED) {
                eval_detail::mixed_channel<D, O, false>(t, plan, cell, xr, base, off,
                                                        static_cast<const float*>(t.ctrl), nullptr, out, out_f32, o0,
                                                        1, 0);
            } else {
                const double* __restrict__ cp = static_cast<const double*>(t.ctrl);
                double acc = 0;
#pragma unroll
                for (int r = 0; r < ROWS; ++r) {
                    int64_t o = 0;
                    double wr = 1;
                    int rem = r;
#pragma unroll
                    for (int d = D - 2; d >= 0; --d) {
                        const int i = rem % W;
                        rem /= W;
                        o += off[d][i];
                        wr *= base[d][i];
                    }
                    double s = 0;
#pragma unroll
                    for (int i = 0; i < W; ++i) s += base[D - 1][i] * __ldg(cp + o + off[D - 1][i]);
                    acc += wr * s;
                }
                if (out_f32)
                    static_cast<float*>(out)[o0] = static_cast<float>(acc);
                else
                    static_cast<double*>(out)[o0] = acc;
            }
        }
    }
}

int proxy_grid(int64_t npts) {
    int64_t g = (npts + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    return static_cast<int>(g < 1 ? 1 : g);
}

template <int D, int O>
cudaError_t build_do(const TableDev& t, bool mixed, const double* coords, int64_t npts, int64_t* cells, void* xr,
                     void* base, cudaStream_t s) {
    if (mixed)
        proxy_build_kernel<D, O, true><<<proxy_grid(npts), 256, 0, s>>>(t, coords, npts, cells, xr, base);
    else
        proxy_build_kernel<D, O, false><<<proxy_grid(npts), 256, 0, s>>>(t, coords, npts, cells, xr, base);
    note_launch();
    return cudaGetLastError();
}

template <int D, int O>
cudaError_t eval_do(const TableDev* tables, int ntables, bool mixed, int64_t npts, const int64_t* cells,
                    const void* xr, const void* base, const DerivPlan& plan, void* out, int out_f32, cudaStream_t s) {
    if (mixed)
        proxy_eval_kernel<D, O, true>
            <<<proxy_grid(npts), 256, 0, s>>>(tables, ntables, npts, cells, xr, base, plan, out, out_f32);
    else
        proxy_eval_kernel<D, O, false>
            <<<proxy_grid(npts), 256, 0, s>>>(tables, ntables, npts, cells, xr, base, plan, out, out_f32);
    note_launch();
    return cudaGetLastError();
}

template <int D>
cudaError_t build_d(const TableDev& t, int order, bool mixed, const double* coords, int64_t npts, int64_t* cells,
                    void* xr, void* base, cudaStream_t s) {
    switch (order) {
        case 0: return build_do<D, 0>(t, mixed, coords, npts, cells, xr, base, s);
        case 1: return build_do<D, 1>(t, mixed, coords, npts, cells, xr, base, s);
        case 2: return build_do<D, 2>(t, mixed, coords, npts, cells, xr, base, s);
        case 3: return build_do<D, 3>(t, mixed, coords, npts, cells, xr, base, s);
        case 4: return build_do<D, 4>(t, mixed, coords, npts, cells, xr, base, s);
        case 5: return build_do<D, 5>(t, mixed, coords, npts, cells, xr, base, s);
        case 6: return build_do<D, 6>(t, mixed, coords, npts, cells, xr, base, s);
        case 7: return build_do<D, 7>(t, mixed, coords, npts, cells, xr, base, s);
    }
    return cudaErrorInvalidValue;
}

template <int D>
cudaError_t eval_d(const TableDev* tables, int ntables, int order, bool mixed, int64_t npts, const int64_t* cells,
                   const void* xr, const void* base, const DerivPlan& plan, void* out, int out_f32, cudaStream_t s) {
    switch (order) {
        case 0: return eval_do<D, 0>(tables, ntables, mixed, npts, cells, xr, base, plan, out, out_f32, s);
        case 1: return eval_do<D, 1>(tables, ntables, mixed, npts, cells, xr, base, plan, out, out_f32, s);
        case 2: return eval_do<D, 2>(tables, ntables, mixed, npts, cells, xr, base, plan, out, out_f32, s);
        case 3: return eval_do<D, 3>(tables, ntables, mixed, npts, cells, xr, base, plan, out, out_f32, s);
        case 4: return eval_do<D, 4>(tables, ntables, mixed, npts, cells, xr, base, plan, out, out_f32, s);
        case 5: return eval_do<D, 5>(tables, ntables, mixed, npts, cells, xr, base, plan, out, out_f32, s);
        case 6: return eval_do<D, 6>(tables, ntables, mixed, npts, cells, xr, base, plan, out, out_f32, s);
        case 7: return eval_do<D, 7>(tables, ntables, mixed, npts, cells, xr, base, plan, out, out_f32, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_proxy_build(const TableDev& t, bool mixed, const double* coords, int64_t npts, int64_t* cells,
                               void* xr, void* base, cudaStream_t s) {
    if (npts <= 0) return cudaSuccess;
    switch (t.dim) {
        case 1: return build_d<1>(t, t.order, mixed, coords, npts, cells, xr, base, s);
        case 2: return build_d<2>(t, t.order, mixed, coords, npts, cells, xr, base, s);
        case 3: return build_d<3>(t, t.order, mixed, coords, npts, cells, xr, base, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_proxy_eval(const TableDev* tables, int ntables, int dim, int order, bool mixed, int64_t npts,
                              const int64_t* cells, const void* xr, const void* base, const DerivPlan& plan, void* out,
                              int out_f32, cudaStream_t s) {
    if (npts <= 0 || ntables <= 0) return cudaSuccess;
    switch (dim) {
        case 1: return eval_d<1>(tables, ntables, order, mixed, npts, cells, xr, base, plan, out, out_f32, s);
        case 2: return eval_d<2>(tables, ntables, order, mixed, npts, cells, xr, base, plan, out, out_f32, s);
        case 3: return eval_d<3>(tables, ntables, order, mixed, npts, cells, xr, base, plan, out, out_f32, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace intp_gb300
