// Instantiations of the direct evaluation kernel: mixed form (FP32 basis and contraction), D = 3;
// orders 6 and 7 live in eval_f32_d3_o67.cu, D = 4 in eval_f32_d4.cu.
#include "eval_impl.cuh"

namespace intp_gb300 {

cudaError_t launch_eval_direct_f32_d3_o67(const TableDev& t, const double* coords, int64_t npts,
                                          const DerivPlan& plan, void* out, bool out_f32, cudaStream_t s);

namespace {

using eval_detail::eval_direct_kernel;

template <int D, int O>
cudaError_t launch_do(const TableDev& t, const double* coords, int64_t npts, const DerivPlan& plan,
                      void* out, bool out_f32, cudaStream_t s) {
    const int block = 128;
    int64_t g = (npts + block - 1) / block;
    if (g > 152 * 32) g = 152 * 32;
    eval_direct_kernel<D, O, true><<<static_cast<int>(g), block, 0, s>>>(t, coords, npts, plan, out,
                                                                      out_f32 ? 1 : 0);
    note_launch();
    return cudaGetLastError();
}

template <int D>
cudaError_t launch_d(const TableDev& t, const double* coords, int64_t npts, const DerivPlan& plan,
                     void* out, bool out_f32, cudaStream_t s) {
    switch (t.order) {
        case 0: return launch_do<D, 0>(t, coords, npts, plan, out, out_f32, s);
        case 1: return launch_do<D, 1>(t, coords, npts, plan, out, out_f32, s);
        case 2: return launch_do<D, 2>(t, coords, npts, plan, out, out_f32, s);
        case 3: return launch_do<D, 3>(t, coords, npts, plan, out, out_f32, s);
        case 4: return launch_do<D, 4>(t, coords, npts, plan, out, out_f32, s);
        case 5: return launch_do<D, 5>(t, coords, npts, plan, out, out_f32, s);
        case 6:
        case 7: return launch_eval_direct_f32_d3_o67(t, coords, npts, plan, out, out_f32, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_eval_direct_f32_d4(const TableDev& t, const double* coords, int64_t npts, const DerivPlan& plan,
                                     void* out, bool out_f32, cudaStream_t s);

cudaError_t launch_eval_direct_f32_d34(const TableDev& t, const double* coords, int64_t npts,
                                       const DerivPlan& plan, void* out, bool out_f32,
                                       cudaStream_t s) {
    switch (t.dim) {
        case 3: return launch_d<3>(t, coords, npts, plan, out, out_f32, s);
        case 4: return launch_eval_direct_f32_d4(t, coords, npts, plan, out, out_f32, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace intp_gb300
