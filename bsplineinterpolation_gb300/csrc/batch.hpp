// Work lists shared by the batched-table host code (batch.cu) and the batched
// evaluation kernels (batch_eval_d*.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "device_common.cuh"

namespace intp_gb300 {

// Up to 32 lines of one table along one axis, solved by one warp (lane l
// takes line line0 + l). Line l of axis a starts at element o*n*S + t with
// o = l / S, t = l % S, where S is the axis stride; consecutive lines of a
// strided axis (S > 1) are adjacent in memory, so the warp's accesses
// coalesce. Lines of the contiguous axis (S = 1) are staged in shared memory
// when `staged` is set.
struct SolveItem {
    int32_t table;
    int16_t axis;
    int8_t staged;
    int8_t pad8;
    int32_t rows;
    int32_t pad;
    int64_t line0;
};

// A run of at most kChunkElems consecutive control points of one table.
struct ChunkItem {
    int32_t table;
    int32_t len;
    int64_t start;  // element index within the table
};

// A run of query points of one table, evaluated by one CTA.
struct EvalItem {
    int32_t table;
    int32_t count;
    int64_t coord_off;  // first coordinate (in doubles) of the run
    int64_t out_pt;     // global index of the run's first point
};

// Evaluates the items of one (dim, order) class: tables[] are the batch's
// device descriptors (control points bound).
cudaError_t launch_batch_eval(int dim, int order, bool mixed, const TableDev* tables, const EvalItem* items,
                              int64_t nitems, const double* coords, const DerivPlan& plan, void* out, bool out_f32,
                              cudaStream_t s);

}  // namespace intp_gb300
