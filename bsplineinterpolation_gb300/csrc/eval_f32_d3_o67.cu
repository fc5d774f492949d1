// Instantiations of the direct evaluation kernel: mixed form (FP32 basis and contraction), D = 3,
// orders 6 and 7 (their own translation unit so that they compile in parallel with the rest).
#include "eval_impl.cuh"

namespace intp_gb300 {

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

}  // namespace

cudaError_t launch_eval_direct_f32_d3_o67(const TableDev& t, const double* coords, int64_t npts,
                                          const DerivPlan& plan, void* out, bool out_f32, cudaStream_t s) {
    return t.order == 6 ? launch_do<3, 6>(t, coords, npts, plan, out, out_f32, s)
                        : launch_do<3, 7>(t, coords, npts, plan, out, out_f32, s);
}

}  // namespace intp_gb300
