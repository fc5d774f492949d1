// Kernel launchers shared between the CUDA translation units and the C-ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "device_common.cuh"
#include "dw.cuh"

namespace intp_gb300 {

// Counts kernel launches made by the library (reported by intp_launch_count).
void note_launch(int count = 1);

struct ShiftDesc {
    int dim;
    int64_t total;     // mesh points
    int64_t channels;  // values per point (source channel fastest, destination channel-major)
    int64_t n[4];
    int64_t shift[4];
    int64_t stride[4];
};

// direct evaluation (eval_misc.cu dispatching to eval_f32_* / eval_f64_*)
cudaError_t launch_eval_direct(const TableDev& t, bool mixed, const double* coords, int64_t npts,
                               const DerivPlan& plan, void* out, bool out_f32, cudaStream_t s);
// Binned evaluation of the mixed form (bin_host.cu); `chunk` queries per round.
// tmap: TMA maps of the control points and of their remainders (the second
// used when t.ctrl_lo is set) with the tile as their box (NULL: the tiles
// are staged with element copies).
cudaError_t run_binned_eval(const TableDev& t, const BinGeom& g, const CUtensorMap* tmap, const double* coords,
                            int64_t npts, const DerivPlan& plan, void* out, bool out_f32, int64_t chunk,
                            cudaStream_t s);
// One chunk's counting sort by bucket into caller-provided scratch: blkcount
// and blkoffset hold nbuckets * nblk entries, tile_sum ceil(that / 4096); rec
// holds n records of bin_record_words(D) words each, in bucket order. Needs
// n <= nblk * 2^20. Returns the slice of input queries each sort CTA took
// (for the evaluation).
cudaError_t bin_sort_chunk(const TableDev& t, const BinGeom& g, const double* coords, int64_t n, int nblk,
                           uint32_t* blkcount, uint32_t* blkoffset, uint32_t* tile_sum, uint32_t* rec, int64_t* slice,
                           cudaStream_t s);
int bin_record_words(int dim);
// (launch_bin_eval_*: `grid` is the SM count; the launchers place as many
// evaluation CTAs per SM as fit.)
// Knot spans (npts x D int64, device memory) of the binned path: the locate
// kernel of the binned evaluation, its records decoded (diagnostics).
cudaError_t binned_span_readout(const TableDev& t, const BinGeom& g, const double* coords, int64_t npts,
                                int64_t* cells, cudaStream_t s);
cudaError_t launch_bin_eval_d12(const TableDev&, const BinGeom&, const CUtensorMap* tmap, const uint32_t* blkoffset,
                                int nblk, int64_t slice, const uint32_t* rec, int64_t n, const DerivPlan&, void* out,
                                bool out_f32, int grid, cudaStream_t);
cudaError_t launch_bin_eval_d3(const TableDev&, const BinGeom&, const CUtensorMap* tmap, const uint32_t* blkoffset,
                               int nblk, int64_t slice, const uint32_t* rec, int64_t n, const DerivPlan&, void* out,
                               bool out_f32, int grid, cudaStream_t);
// Read and clear the device error flag of the binned evaluation units.
int take_device_error_bin_d12(cudaStream_t s);
int take_device_error_bin_d3(cudaStream_t s);
// Diagnostics: probes of the binned evaluation's tile wait (0 = normal wait).
cudaError_t set_wait_probes_bin_d12(uint32_t probes);
cudaError_t set_wait_probes_bin_d3(uint32_t probes);
// Caps the warm-up of the warp-segmented line solves (test hook; -1: none).
cudaError_t set_warm_cap_solve(int rows);
cudaError_t set_warm_cap_batch(int rows);
// Bucket geometry of the binned evaluation for a table: compile-time bucket
// sizes per dimension (bucket_log2); smem_buckets = 0 when the table has too
// many buckets or too many knots for the binned path.
BinGeom make_bin_geom(const TableDev& t);

cudaError_t launch_locate(const TableDev& t, const double* coords, int64_t npts, int64_t* cells,
                          double* wrapped, cudaStream_t s);
cudaError_t launch_range_check(const TableDev& t, const double* coords, int64_t npts,
                               unsigned long long* first_bad, cudaStream_t s);

// solve (solve_kernels.cu)
// Band / cyclic-band solves of every line along one axis with the factor's
// lower / upper bands, inverse diagonal and cyclic corner blocks.
// Rows clo .. chi-1 of the factor are identical to row clo (taken from
// registers in those rows; clo = chi: none).
cudaError_t launch_line_solve_f64(double* x, int64_t n, int64_t S, int64_t nlines, int p, int q, bool cyclic,
                                  const double* lower, const double* upper, const double* dinv, const double* bottom,
                                  const double* right, cudaStream_t s, int64_t clo = 0, int64_t chi = 0,
                                  int64_t zside = INT64_MAX);
cudaError_t launch_line_solve_f32(float* x, int64_t n, int64_t S, int64_t nlines, int p, int q, bool cyclic,
                                  const float* lower, const float* upper, const float* dinv, const float* bottom,
                                  const float* right, cudaStream_t s, int64_t clo = 0, int64_t chi = 0,
                                  int64_t zside = INT64_MAX);
// Evaluation proxies (proxy.cu): per point and axis its span (cells), offset
// (xr: FP64 coordinate, or FP32 local offset for mixed tables) and O+1
// value weights (base), then the values of ntables tables (a device array of
// descriptors) at every point, out[i * ntables + j].
cudaError_t launch_proxy_build(const TableDev& t, bool mixed, const double* coords, int64_t npts, int64_t* cells,
                               void* xr, void* base, cudaStream_t s);
cudaError_t launch_proxy_eval(const TableDev* tables, int ntables, int dim, int order, bool mixed, int64_t npts,
                              const int64_t* cells, const void* xr, const void* base, const DerivPlan& plan, void* out,
                              int out_f32, cudaStream_t s);
// The mixed form's double-word line solve (same substitution as the FP32 and
// FP64 solves, R = DW), its right-hand side (the shifted values split into
// double-words) and the split of its solution into the table's two FP32
// arrays.
cudaError_t launch_line_solve_dw(DW* x, int64_t n, int64_t S, int64_t nlines, int p, int q, bool cyclic,
                                 const DW* lower, const DW* upper, const DW* dinv, const DW* bottom, const DW* right,
                                 cudaStream_t s, int64_t clo = 0, int64_t chi = 0, int64_t zside = INT64_MAX);
cudaError_t launch_shift_copy_f64_dw(const double* src, DW* dst, const ShiftDesc& sd, cudaStream_t s);
cudaError_t launch_dw_unpack(const DW* w, float* hi, float* lo, int64_t n, cudaStream_t s);
cudaError_t launch_shift_copy_f64_f64(const double* src, double* dst, const ShiftDesc& sd,
                                      cudaStream_t s);
// FP32 copy; with dst_lo the double-float split (dst + dst_lo = the value),
// the high part written to dst2 as well.
cudaError_t launch_shift_copy_f64_f32(const double* src, float* dst, float* dst_lo, float* dst2, const ShiftDesc& sd,
                                      cudaStream_t s);
// Reads and clears the device error flag set by a kernel whose bounded wait
// ran out (0 = none).
int take_device_error(cudaStream_t s);

}  // namespace intp_gb300
