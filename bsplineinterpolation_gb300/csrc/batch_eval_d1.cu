// Instantiations of the batched evaluation kernel, D = 1 (mixed and FP64 forms).
#include "batch_eval_impl.cuh"

namespace intp_gb300 {

cudaError_t launch_batch_eval_d1(int order, bool mixed, const TableDev* tables, const EvalItem* items, int64_t nitems,
                                 const double* coords, const DerivPlan& plan, void* out, bool out_f32, cudaStream_t s) {
    if (mixed) return batch_detail::launch_d<1, true>(order, tables, items, nitems, coords, plan, out, out_f32, s);
    return batch_detail::launch_d<1, false>(order, tables, items, nitems, coords, plan, out, out_f32, s);
}

cudaError_t launch_batch_eval(int dim, int order, bool mixed, const TableDev* tables, const EvalItem* items,
                              int64_t nitems, const double* coords, const DerivPlan& plan, void* out, bool out_f32,
                              cudaStream_t s) {
    if (nitems <= 0) return cudaSuccess;
    switch (dim) {
        case 1: return launch_batch_eval_d1(order, mixed, tables, items, nitems, coords, plan, out, out_f32, s);
        case 2: return launch_batch_eval_d2(order, mixed, tables, items, nitems, coords, plan, out, out_f32, s);
        case 3: return launch_batch_eval_d3(order, mixed, tables, items, nitems, coords, plan, out, out_f32, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace intp_gb300
