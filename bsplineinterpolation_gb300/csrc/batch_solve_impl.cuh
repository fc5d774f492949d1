// The batched line-solve kernel, one instance per (element type, band class):
// a class is a (band width, cyclic) pair, and a work item's class fixes which
// substitution it runs. Each instance holds the code of its one class only,
// so its registers and instruction footprint are those of that class and not
// of the widest band a batch may hold; a pass launches one instance per class
// present. Included by batch_solve_{f32,dw,f64}.cu, one element type each.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <utility>

#include "batch.hpp"
#include "launch.hpp"
#include "solve_line.cuh"
#include "table_pack.hpp"

namespace intp_gb300 {
namespace batch_solve_detail {

template <class R>
__device__ __forceinline__ FactorView<R> factor_view(const AxisFactorDev& f, int64_t n);

template <>
__device__ __forceinline__ FactorView<float> factor_view<float>(const AxisFactorDev& f, int64_t n) {
    return FactorView<float>{n, f.lowerf, f.upperf, f.dinvf, f.bottomf, f.rightf, f.clo32, f.chi32, f.zside32};
}

template <>
__device__ __forceinline__ FactorView<double> factor_view<double>(const AxisFactorDev& f, int64_t n) {
    return FactorView<double>{n, f.lower, f.upper, f.dinv, f.bottom, f.right, f.clo, f.chi, f.zside};
}

template <>
__device__ __forceinline__ FactorView<DW> factor_view<DW>(const AxisFactorDev& f, int64_t n) {
    return FactorView<DW>{n, f.lowerw, f.upperw, f.dinvw, f.bottomw, f.rightw, f.clo, f.chi, f.zside};
}

__device__ __forceinline__ bool selected(int sel, int refine) {
    return sel == kBatchSelAll || (sel == kBatchSelPlain ? refine == 0 : refine > 0);
}

// Lines are walked in chunks of this many elements (registers per lane; the
// next chunk's strided loads are held in registers too).
template <class R>
constexpr int chunk_of() {
    return sizeof(R) == 4 ? 16 : 8;
}

// A line of at least this many elements that is a warp's only line is solved
// by the whole warp (solve_line_warp).
constexpr int64_t kWarpLineMin = 128;

// Warm-up rows of the warp-segmented substitution: enough for the zero
// state's error to fall below the last bit in FP32 / FP64.
template <class R>
constexpr int warm_rows() {
    return sizeof(R) == 4 ? 64 : 128;
}

// Contiguous lines: chunks through a double per-warp stage, the next
// chunk's rows in flight while one is solved.
template <class R>
using ContigIo = WarpContigChunksPF<R, chunk_of<R>()>;

// The work of one item (up to 32 lines of one table and axis, band P = Q,
// cyclic or not) for one warp. `sel` picks the tables of a mixed batch.
template <class R, int P, bool CYC>
__device__ __forceinline__ void solve_item(R* __restrict__ data, const SolveItem& it, R* tile,
                                           const TableDev* __restrict__ tables,
                                           const AxisFactorDev* __restrict__ fac, const int64_t* __restrict__ off,
                                           const int32_t* __restrict__ refine, int sel) {
    if (!selected(sel, refine[it.table])) return;
    const int lane = threadIdx.x;
    const TableDev& t = tables[it.table];
    const AxisDev& ax = t.ax[it.axis];
    const int64_t n = ax.n, S = ax.stride;
    const FactorView<R> fv = factor_view<R>(fac[it.table * kBatchMaxDim + it.axis], n);
    R* base = data + off[it.table] + it.chan * t.chan_stride;
    if (it.contig) {
        // S == 1: lines line0 .. line0+rows-1 are one contiguous run of
        // rows*n; each chunk moves through the warp's [32][chunk+1] stages
        // (all lanes take part, lane l owning line line0 + l)
        R* x = base + it.line0 * n;
        if (it.rows == 1 && n >= kWarpLineMin)
            solve_line_warp<R, P, P, CYC, warm_rows<R>(), true>(fv, LineRef<R>{x, 1}, lane);
        else
            solve_line_chunked<R, P, P, CYC, chunk_of<R>()>(fv, ContigIo<R>{x, n, it.rows, tile, lane});
        return;
    }
    if (lane < it.rows) {
        const int64_t l = it.line0 + lane;
        const int64_t o = l / S, tt = l - o * S;
        solve_line_chunked<R, P, P, CYC, chunk_of<R>()>(fv, StridedChunks<R>{base + o * n * S + tt, S});
    }
}

// One warp per CTA. PERSIST: a grid of a few warps per SM drains the list
// through an atomic counter (longest lines first), else one CTA per item.
template <class R, bool PERSIST, int P, bool CYC>
__global__ void __launch_bounds__(32, 16) solve_kernel(R* __restrict__ data, const SolveItem* __restrict__ items,
                                                   int64_t nitems, unsigned int* __restrict__ counter,
                                                   const TableDev* __restrict__ tables,
                                                   const AxisFactorDev* __restrict__ fac,
                                                   const int64_t* __restrict__ off,
                                                   const int32_t* __restrict__ refine, int sel) {
    __shared__ __align__(16) R tile[ContigIo<R>::kStageElems];
    if constexpr (!PERSIST) {
        solve_item<R, P, CYC>(data, items[blockIdx.x], tile, tables, fac, off, refine, sel);
    } else {
        for (;;) {
            unsigned int idx = 0;
            if (threadIdx.x == 0) idx = atomicAdd(counter, 1u);
            idx = __shfl_sync(0xFFFFFFFFu, idx, 0);
            if (static_cast<int64_t>(idx) >= nitems) return;
            solve_item<R, P, CYC>(data, items[idx], tile, tables, fac, off, refine, sel);
            __syncwarp();
        }
    }
}

template <class R, bool PERSIST>
using SolveKernelFn = void (*)(R*, const SolveItem*, int64_t, unsigned int*, const TableDev*, const AxisFactorDev*,
                               const int64_t*, const int32_t*, int);

template <class R, bool PERSIST, int C>
constexpr SolveKernelFn<R, PERSIST> class_kernel() {
    if constexpr (C <= kBatchMaxBand)
        return solve_kernel<R, PERSIST, C, false>;
    else
        return solve_kernel<R, PERSIST, C - kBatchMaxBand - 1, true>;
}

template <class R, bool PERSIST, int... C>
SolveKernelFn<R, PERSIST> kernel_of(int cls, std::integer_sequence<int, C...>) {
    static const SolveKernelFn<R, PERSIST> table[] = {class_kernel<R, PERSIST, C>()...};
    return table[cls];
}

template <class R>
cudaError_t launch(R* data, int cls, const BatchSolveLaunch& a, cudaStream_t s) {
    if (a.nitems <= 0) return cudaSuccess;
    if (cls < 0 || cls >= kBatchClasses) return cudaErrorInvalidValue;
    const auto seq = std::make_integer_sequence<int, kBatchClasses>{};
    if (a.persistent) {
        auto k = kernel_of<R, true>(cls, seq);
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 32, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
        const int64_t grid = std::min<int64_t>(a.nitems, static_cast<int64_t>(per_sm) * a.sm_count);
        k<<<static_cast<unsigned>(grid), 32, 0, s>>>(data, a.items, a.nitems, a.counter, a.tables, a.fac, a.off,
                                                      a.refine, a.sel);
    } else {
        auto k = kernel_of<R, false>(cls, seq);
        k<<<static_cast<unsigned>(a.nitems), 32, 0, s>>>(data, a.items, a.nitems, nullptr, a.tables, a.fac, a.off,
                                                         a.refine, a.sel);
    }
    note_launch();
    return cudaGetLastError();
}

}  // namespace batch_solve_detail
}  // namespace intp_gb300

// The warm-up cap test hook of this translation unit's solve_line_warp, and
// the launcher for one element type.
#define INTP_DEFINE_BATCH_SOLVE(R, SUFFIX)                                                            \
    namespace intp_gb300 {                                                                            \
    INTP_DEFINE_WARM_CAP_SETTER(set_warm_cap_batch_##SUFFIX)                                          \
    cudaError_t launch_batch_solve(R* data, int cls, const BatchSolveLaunch& a, cudaStream_t s) {     \
        return batch_solve_detail::launch<R>(data, cls, a, s);                                       \
    }                                                                                                 \
    }
