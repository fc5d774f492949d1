// Work lists shared by the batched-table host code (batch.cu) and the batched
// evaluation kernels (batch_eval_d*.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "device_common.cuh"
#include "dw.cuh"

namespace intp_gb300 {

struct AxisFactorDev;

constexpr int kBatchMaxDim = 3;

// Band classes of the line solves: non-cyclic bands p = q = 0..kBatchMaxBand
// are classes 0..kBatchMaxBand, cyclic bands p = q = 0..kBatchMaxCyclicBand
// follow them. Each class has its own kernel instance.
constexpr int kBatchMaxBand = 6, kBatchMaxCyclicBand = 3;
constexpr int kBatchClasses = kBatchMaxBand + 1 + kBatchMaxCyclicBand + 1;
inline int batch_band_class(int p, bool cyclic) { return cyclic ? kBatchMaxBand + 1 + p : p; }

// Tables a solve launch works on (mixed batches): every table, the tables
// solved in FP32 (refine = 0), or the ones solved in double-word arithmetic.
constexpr int kBatchSelAll = -1, kBatchSelPlain = -2, kBatchSelDW = -3;


// Up to 32 lines of one table along one axis, solved by one warp (lane l
// takes line line0 + l). Line l of axis a starts at element o*n*S + t with
// o = l / S, t = l % S, where S is the axis stride; consecutive lines of a
// strided axis (S > 1) are adjacent in memory, so the warp's accesses
// coalesce. Lines of the contiguous axis (S = 1, `contig` set) move chunk by
// chunk through a per-warp shared-memory transpose. A vector-valued table
// stores each channel's control points as one mesh (channel ch at
// ch * chan_stride); an item covers lines of one channel.
struct SolveItem {
    int32_t table;
    int16_t axis;
    int8_t contig;
    int8_t pad8;
    int32_t rows;
    int32_t chan;
    int64_t line0;
};

// A run of at most kChunkElems consecutive control points of one table.
struct ChunkItem {
    int32_t table;
    int32_t len;
    int64_t start;  // element index within the table
};

// A run of query points of one table, evaluated by one CTA. Point i of the
// run writes its K outputs of every channel ch at out_elem + (i*K + k)*C + ch.
struct EvalItem {
    int32_t table;
    int32_t count;
    int64_t coord_off;  // first coordinate (in doubles) of the run
    int64_t out_elem;   // first output element of the run
};

// One launch of the batched line solves: the work items of one pass and one
// band class, and the batch's device arrays.
struct BatchSolveLaunch {
    const SolveItem* items;
    int64_t nitems;
    unsigned int* counter;  // work counter (persistent launches)
    const TableDev* tables;
    const AxisFactorDev* fac;  // [table * kBatchMaxDim + axis]
    const int64_t* off;        // control-point offset of each table
    const int32_t* refine;     // per table: 0 FP32 solve, > 0 double-word solve
    int sel;                   // kBatchSel*
    bool persistent;           // a grid of a few warps per SM drains an atomic work queue
    int sm_count;
};

// Solves the items of one band class in place (batch_solve_{f32,dw,f64}.cu).
cudaError_t launch_batch_solve(float* data, int cls, const BatchSolveLaunch& a, cudaStream_t s);
cudaError_t launch_batch_solve(DW* data, int cls, const BatchSolveLaunch& a, cudaStream_t s);
cudaError_t launch_batch_solve(double* data, int cls, const BatchSolveLaunch& a, cudaStream_t s);

// Test hook: caps the warm-up rows of the warp-segmented substitution in
// each of those translation units (< 0 restores the default).
cudaError_t set_warm_cap_batch_f32(int rows);
cudaError_t set_warm_cap_batch_dw(int rows);
cudaError_t set_warm_cap_batch_f64(int rows);

// Evaluates the items of one (dim, order) class: tables[] are the batch's
// device descriptors (control points bound).
cudaError_t launch_batch_eval(int dim, int order, bool mixed, const TableDev* tables, const EvalItem* items,
                              int64_t nitems, const double* coords, const DerivPlan& plan, void* out, bool out_f32,
                              cudaStream_t s);

}  // namespace intp_gb300
