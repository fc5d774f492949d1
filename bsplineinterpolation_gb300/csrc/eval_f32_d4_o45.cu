// Instantiations of the direct evaluation kernel: mixed form (FP32 basis and
// contraction), D = 4, orders 4, 5. The 4D orders are split over several
// translation units: a single one holding all eight compiled for minutes.
#include "eval_impl.cuh"

namespace intp_gb300 {

namespace {

template <int O>
cudaError_t launch_do(const TableDev& t, const double* coords, int64_t npts, const DerivPlan& plan, void* out,
                      bool out_f32, cudaStream_t s) {
    const int block = 128;
    int64_t g = (npts + block - 1) / block;
    if (g > 152 * 32) g = 152 * 32;
    eval_detail::eval_direct_kernel<4, O, true>
        <<<static_cast<int>(g), block, 0, s>>>(t, coords, npts, plan, out, out_f32 ? 1 : 0);
    note_launch();
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_eval_direct_f32_d4_o45(const TableDev& t, const double* coords, int64_t npts, const DerivPlan& plan, void* out,
                                          bool out_f32, cudaStream_t s) {
    switch (t.order) {
        case 4: return launch_do<4>(t, coords, npts, plan, out, out_f32, s);
        case 5: return launch_do<5>(t, coords, npts, plan, out, out_f32, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace intp_gb300
