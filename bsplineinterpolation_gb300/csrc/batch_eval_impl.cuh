// Batched evaluation kernel: one CTA per run of query points of one table
// (EvalItem), one thread per point, the per-point code of the direct kernel
// (eval_point) on the table's descriptor staged in shared memory.
#pragma once

#include "batch.hpp"
#include "eval_impl.cuh"

namespace intp_gb300 {
namespace batch_detail {

constexpr int kBatchEvalThreads = 128;

// LO: the plan has derivative outputs (mixed tables then contract with the
// control points' remainders); value-only plans run an instance without that
// code, with fewer registers.
template <int D, int O, bool MIXED, bool LO>
__global__ void __launch_bounds__(kBatchEvalThreads) batch_eval_kernel(const TableDev* __restrict__ tables,
                                                                       const EvalItem* __restrict__ items,
                                                                       int64_t nitems, const double* __restrict__ coords,
                                                                       DerivPlan plan, void* __restrict__ out,
                                                                       int out_f32) {
    __shared__ TableDev sh_t;
    for (int64_t w = blockIdx.x; w < nitems; w += gridDim.x) {
        const EvalItem it = items[w];
        __syncthreads();
        {
            const int* src = reinterpret_cast<const int*>(tables + it.table);
            int* dst = reinterpret_cast<int*>(&sh_t);
            constexpr int nwords = static_cast<int>(sizeof(TableDev) / sizeof(int));
            for (int i = threadIdx.x; i < nwords; i += blockDim.x) dst[i] = src[i];
        }
        __syncthreads();
        const double* xs = coords + it.coord_off;
        void* o = out_f32 ? static_cast<void*>(static_cast<float*>(out) + it.out_elem)
                          : static_cast<void*>(static_cast<double*>(out) + it.out_elem);
        for (int i = threadIdx.x; i < it.count; i += blockDim.x)
            eval_detail::eval_point<D, O, MIXED, LO>(sh_t, xs + static_cast<int64_t>(i) * D, plan, o, out_f32,
                                                 static_cast<int64_t>(i) * plan.k);
    }
}

template <int D, int O, bool MIXED>
cudaError_t launch_one(const TableDev* tables, const EvalItem* items, int64_t nitems, const double* coords,
                       const DerivPlan& plan, void* out, bool out_f32, cudaStream_t s) {
    const int64_t grid = nitems < 152 * 64 ? nitems : 152 * 64;
    if (MIXED && plan.has_deriv)
        batch_eval_kernel<D, O, MIXED, true><<<static_cast<unsigned>(grid), kBatchEvalThreads, 0, s>>>(
            tables, items, nitems, coords, plan, out, out_f32 ? 1 : 0);
    else
        batch_eval_kernel<D, O, MIXED, false><<<static_cast<unsigned>(grid), kBatchEvalThreads, 0, s>>>(
            tables, items, nitems, coords, plan, out, out_f32 ? 1 : 0);
    note_launch();
    return cudaGetLastError();
}

template <int D, bool MIXED>
cudaError_t launch_d(int order, const TableDev* tables, const EvalItem* items, int64_t nitems, const double* coords,
                     const DerivPlan& plan, void* out, bool out_f32, cudaStream_t s) {
    switch (order) {
        case 0: return launch_one<D, 0, MIXED>(tables, items, nitems, coords, plan, out, out_f32, s);
        case 1: return launch_one<D, 1, MIXED>(tables, items, nitems, coords, plan, out, out_f32, s);
        case 2: return launch_one<D, 2, MIXED>(tables, items, nitems, coords, plan, out, out_f32, s);
        case 3: return launch_one<D, 3, MIXED>(tables, items, nitems, coords, plan, out, out_f32, s);
        case 4: return launch_one<D, 4, MIXED>(tables, items, nitems, coords, plan, out, out_f32, s);
        case 5: return launch_one<D, 5, MIXED>(tables, items, nitems, coords, plan, out, out_f32, s);
        case 6: return launch_one<D, 6, MIXED>(tables, items, nitems, coords, plan, out, out_f32, s);
        case 7: return launch_one<D, 7, MIXED>(tables, items, nitems, coords, plan, out, out_f32, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace batch_detail

// Launchers of one dimension (batch_eval_d*.cu).
cudaError_t launch_batch_eval_d1(int order, bool mixed, const TableDev* tables, const EvalItem* items, int64_t nitems,
                                 const double* coords, const DerivPlan& plan, void* out, bool out_f32, cudaStream_t s);
cudaError_t launch_batch_eval_d2(int order, bool mixed, const TableDev* tables, const EvalItem* items, int64_t nitems,
                                 const double* coords, const DerivPlan& plan, void* out, bool out_f32, cudaStream_t s);
cudaError_t launch_batch_eval_d3(int order, bool mixed, const TableDev* tables, const EvalItem* items, int64_t nitems,
                                 const double* coords, const DerivPlan& plan, void* out, bool out_f32, cudaStream_t s);

}  // namespace intp_gb300
