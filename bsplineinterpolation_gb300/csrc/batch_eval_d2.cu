// Instantiations of the batched evaluation kernel, D = 2 (mixed and FP64 forms).
#include "batch_eval_impl.cuh"

namespace intp_gb300 {

cudaError_t launch_batch_eval_d2(int order, bool mixed, const TableDev* tables, const EvalItem* items, int64_t nitems,
                                 const double* coords, const DerivPlan& plan, void* out, bool out_f32, cudaStream_t s) {
    if (mixed) return batch_detail::launch_d<2, true>(order, tables, items, nitems, coords, plan, out, out_f32, s);
    return batch_detail::launch_d<2, false>(order, tables, items, nitems, coords, plan, out, out_f32, s);
}

}  // namespace intp_gb300
