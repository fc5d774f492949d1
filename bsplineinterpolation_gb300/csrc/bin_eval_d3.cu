// Instantiations of the binned evaluation kernel (mixed form), D = 3.
#include "bin_impl.cuh"

namespace intp_gb300 {

namespace {

template <int D, int O>
cudaError_t launch_do(const TableDev& t, const BinGeom& g, const CUtensorMap* tmap, const uint32_t* offsets, int nblk,
                      int64_t slice, const uint32_t* rec,
                      int64_t n, const DerivPlan& plan, void* out, bool out_f32, int grid, cudaStream_t s) {
    auto k = bin_detail::eval_kernel<D, O>;
    // the tile, the remainders' tile / sorted records, the records' cells and
    // the cell counters (bin_detail::EvalSmem)
    const size_t smem = bin_detail::EvalSmem<D, O>::kBytes;
    const bool lo = t.ctrl_lo && plan.has_deriv;
    // static + dynamic shared memory may pass 48 KB even when the tile alone
    // does not, so the opt-in limit is set on every launch
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    // FP32 outputs: 1, or 3 when pairs of outputs may leave as 8-byte stores
    const int out_mode = out_f32 ? ((reinterpret_cast<uintptr_t>(out) & 7u) == 0 ? 3 : 1) : 0;
    // a full wave: every SM holds as many evaluation CTAs as fit
    static int per_sm = 0;
    if (per_sm == 0 &&
        (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, bin_detail::kBinThreads, smem) != cudaSuccess ||
         per_sm < 1))
        per_sm = 1;
    grid *= per_sm;  // grid: the SM count
    CUtensorMap none{};
    k<<<grid, bin_detail::kBinThreads, smem, s>>>(t, g, offsets, nblk, slice, rec, n, plan, out, out_mode,
                                                  tmap ? tmap[0] : none, tmap && lo ? tmap[1] : none,
                                                  tmap ? 1 : 0);
    note_launch();
    return cudaGetLastError();
}

template <int D>
cudaError_t launch_d(const TableDev& t, const BinGeom& g, const CUtensorMap* tmap, const uint32_t* offsets, int nblk,
                     int64_t slice, const uint32_t* rec,
                     int64_t n, const DerivPlan& plan, void* out, bool out_f32, int grid, cudaStream_t s) {
    switch (t.order) {
        case 0: return launch_do<D, 0>(t, g, tmap, offsets, nblk, slice, rec, n, plan, out, out_f32, grid, s);
        case 1: return launch_do<D, 1>(t, g, tmap, offsets, nblk, slice, rec, n, plan, out, out_f32, grid, s);
        case 2: return launch_do<D, 2>(t, g, tmap, offsets, nblk, slice, rec, n, plan, out, out_f32, grid, s);
        case 3: return launch_do<D, 3>(t, g, tmap, offsets, nblk, slice, rec, n, plan, out, out_f32, grid, s);
        case 4: return launch_do<D, 4>(t, g, tmap, offsets, nblk, slice, rec, n, plan, out, out_f32, grid, s);
        case 5: return launch_do<D, 5>(t, g, tmap, offsets, nblk, slice, rec, n, plan, out, out_f32, grid, s);
        case 6: return launch_do<D, 6>(t, g, tmap, offsets, nblk, slice, rec, n, plan, out, out_f32, grid, s);
        case 7: return launch_do<D, 7>(t, g, tmap, offsets, nblk, slice, rec, n, plan, out, out_f32, grid, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_bin_eval_d3(const TableDev& t, const BinGeom& g, const CUtensorMap* tmap, const uint32_t* offsets,
                               int nblk, int64_t slice, const uint32_t* rec, int64_t n, const DerivPlan& plan, void* out, bool out_f32, int grid,
                                cudaStream_t s) {
    switch (t.dim) {
        case 3: return launch_d<3>(t, g, tmap, offsets, nblk, slice, rec, n, plan, out, out_f32, grid, s);
    }
    return cudaErrorInvalidValue;
}

INTP_DEFINE_DEVICE_ERROR_READER(take_device_error_bin_d3)
INTP_DEFINE_WAIT_PROBE_SETTER(set_wait_probes_bin_d3)

}  // namespace intp_gb300
