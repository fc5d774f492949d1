// Locate / range-check kernels and the evaluation dispatcher.
#include "eval_impl.cuh"

namespace intp_gb300 {

cudaError_t launch_eval_direct_f64_d12(const TableDev&, const double*, int64_t, const DerivPlan&, void*,
                                       bool, cudaStream_t);
cudaError_t launch_eval_direct_f64_d34(const TableDev&, const double*, int64_t, const DerivPlan&, void*,
                                       bool, cudaStream_t);
cudaError_t launch_eval_direct_f32_d12(const TableDev&, const double*, int64_t, const DerivPlan&, void*,
                                       bool, cudaStream_t);
cudaError_t launch_eval_direct_f32_d34(const TableDev&, const double*, int64_t, const DerivPlan&, void*,
                                       bool, cudaStream_t);

namespace eval_detail {

__global__ void locate_kernel(TableDev t, const double* __restrict__ coords, int64_t npts,
                              int64_t* __restrict__ cells, double* __restrict__ wrapped) {
    const int D = t.dim, O = t.order;
    for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < npts;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        for (int d = 0; d < D; ++d) {
            const AxisDev& a = t.ax[d];
            double x = coords[p * D + d];
            if (a.periodic) x = periodic_wrap(a, x);
            const int64_t h = a.uniform ? uniform_hint(a, x) : static_cast<int64_t>(O);
            cells[p * D + d] = locate_span(a, O, knot_key(x), h);
            if (wrapped) wrapped[p * D + d] = x;
        }
    }
}

// Index of the first point outside the range of a non-periodic axis
// (Interpolation.hpp:482-491), reduced with atomicMin.
__global__ void range_check_kernel(TableDev t, const double* __restrict__ coords, int64_t npts,
                                   unsigned long long* __restrict__ first_bad) {
    const int D = t.dim;
    for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < npts;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        bool bad = false;
        for (int d = 0; d < D; ++d) {
            const AxisDev& a = t.ax[d];
            const double x = coords[p * D + d];
            if (!a.periodic && (x < a.lo || x > a.hi)) bad = true;
        }
        if (bad) atomicMin(first_bad, static_cast<unsigned long long>(p));
    }
}

}  // namespace eval_detail

namespace {

int grid_for(int64_t n, int block, int max_blocks) {
    int64_t g = (n + block - 1) / block;
    if (g > max_blocks) g = max_blocks;
    if (g < 1) g = 1;
    return static_cast<int>(g);
}

}  // namespace

cudaError_t launch_eval_direct(const TableDev& t, bool mixed, const double* coords, int64_t npts,
                               const DerivPlan& plan, void* out, bool out_f32, cudaStream_t s) {
    if (npts <= 0) return cudaSuccess;
    if (t.dim < 1 || t.dim > 4) return cudaErrorInvalidValue;
    if (mixed)
        return t.dim <= 2 ? launch_eval_direct_f32_d12(t, coords, npts, plan, out, out_f32, s)
                          : launch_eval_direct_f32_d34(t, coords, npts, plan, out, out_f32, s);
    return t.dim <= 2 ? launch_eval_direct_f64_d12(t, coords, npts, plan, out, out_f32, s)
                      : launch_eval_direct_f64_d34(t, coords, npts, plan, out, out_f32, s);
}

cudaError_t launch_locate(const TableDev& t, const double* coords, int64_t npts, int64_t* cells,
                          double* wrapped, cudaStream_t s) {
    if (npts <= 0) return cudaSuccess;
    eval_detail::locate_kernel<<<grid_for(npts, 256, 152 * 16), 256, 0, s>>>(t, coords, npts, cells,
                                                                             wrapped);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_range_check(const TableDev& t, const double* coords, int64_t npts,
                               unsigned long long* first_bad, cudaStream_t s) {
    if (npts <= 0) return cudaSuccess;
    eval_detail::range_check_kernel<<<grid_for(npts, 256, 152 * 16), 256, 0, s>>>(t, coords, npts,
                                                                                   first_bad);
    note_launch();
    return cudaGetLastError();
}

}  // namespace intp_gb300
