// Host side of the binned evaluation: bucket geometry, chunk loop, launches
// of the histogram / scan / scatter kernels (the evaluation kernels are
// instantiated in bin_eval_d12.cu and bin_eval_d34.cu).
#include <cuda_runtime.h>

#include <algorithm>

#include "bin_impl.cuh"

namespace intp_gb300 {

cudaError_t launch_bin_eval_d12(const TableDev&, const BinGeom&, const uint32_t*, const uint32_t*,
                                const uint32_t*, const float*, int64_t, int64_t, const DerivPlan&, void*,
                                bool, int, cudaStream_t);
cudaError_t launch_bin_eval_d3(const TableDev&, const BinGeom&, const uint32_t*, const uint32_t*,
                                const uint32_t*, const float*, int64_t, int64_t, const DerivPlan&, void*,
                                bool, int, cudaStream_t);

namespace bin_detail {

// Exclusive scan of counts into offsets[0..nb] and cursor[0..nb) (one block).
__global__ void __launch_bounds__(1024) scan_kernel(const uint32_t* __restrict__ counts, uint32_t* __restrict__ offsets,
                                                    uint32_t* __restrict__ cursor, int64_t nb) {
    __shared__ uint32_t partial[1024];
    const int tid = threadIdx.x;
    const int64_t per = (nb + 1023) / 1024;
    const int64_t b0 = tid * per, b1 = (b0 + per < nb) ? b0 + per : nb;
    uint32_t s = 0;
    for (int64_t b = b0; b < b1; ++b) s += counts[b];
    partial[tid] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const uint32_t v = tid >= off ? partial[tid - off] : 0u;
        __syncthreads();
        partial[tid] += v;
        __syncthreads();
    }
    uint32_t run = tid == 0 ? 0u : partial[tid - 1];
    for (int64_t b = b0; b < b1; ++b) {
        offsets[b] = run;
        cursor[b] = run;
        run += counts[b];
    }
    if (tid == 1023) offsets[nb] = partial[1023];
}

}  // namespace bin_detail

namespace {

constexpr int32_t kSmemBucketLimit = 6144;

int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    }
    return n;
}

template <int D>
cudaError_t launch_hist_scatter(const TableDev& t, const BinGeom& g, const double* coords, int64_t n,
                                uint32_t* counts, uint32_t* offsets, uint32_t* cursor, uint32_t* ridx,
                                uint32_t* rcell, float* ru, int64_t cap, cudaStream_t s) {
    using namespace bin_detail;
    const int grid = sm_count() * 8;
    cudaError_t e = cudaMemsetAsync(counts, 0, static_cast<size_t>(g.nbuckets) * 4, s);
    if (e != cudaSuccess) return e;
    const size_t sm_h = g.smem_buckets > 0 ? static_cast<size_t>(g.smem_buckets) * 4 : 0;
    hist_kernel<D><<<grid, kBinThreads, sm_h, s>>>(t, g, coords, n, counts);
    note_launch();
    scan_kernel<<<1, 1024, 0, s>>>(counts, offsets, cursor, g.nbuckets);
    note_launch();
    scatter_kernel<D><<<grid, kBinThreads, sm_h * 2, s>>>(t, g, coords, n, cursor, ridx, rcell, ru, cap);
    note_launch();
    return cudaGetLastError();
}

}  // namespace

BinGeom make_bin_geom(const TableDev& t, int64_t tile_bytes) {
    BinGeom g{};
    const int D = t.dim, O = t.order;
    g.dim = D;
    int lb[kDevMaxDim] = {0, 0, 0, 0};
    auto tile = [&](const int* l) {
        int64_t e = 1;
        for (int d = 0; d < D; ++d) e *= (int64_t{1} << l[d]) + O;
        return e * 4;
    };
    for (bool grew = true; grew;) {
        grew = false;
        for (int d = D - 1; d >= 0; --d) {
            if ((int64_t{1} << lb[d]) >= t.ax[d].ncells || lb[d] >= 12) continue;
            int trial[kDevMaxDim];
            std::copy(lb, lb + kDevMaxDim, trial);
            ++trial[d];
            if (tile(trial) <= tile_bytes) {
                lb[d] = trial[d];
                grew = true;
            }
        }
    }
    int shift = 0;
    g.nbuckets = 1;
    int32_t stride = 1;
    for (int d = D - 1; d >= 0; --d) {
        g.lb[d] = lb[d];
        g.P[d] = (1 << lb[d]) + O;
        g.nb[d] = static_cast<int32_t>((t.ax[d].ncells + (int64_t{1} << lb[d]) - 1) >> lb[d]);
        g.tstride[d] = stride;
        stride *= g.P[d];
    }
    for (int d = 0; d < D; ++d) {
        g.shift[d] = shift;
        shift += lb[d];
        g.nbuckets *= g.nb[d];
    }
    g.tile_elems = stride;
    g.smem_buckets = g.nbuckets <= kSmemBucketLimit ? static_cast<int32_t>(g.nbuckets) : 0;
    return g;
}

cudaError_t run_binned_eval(const TableDev& t, const BinGeom& g, const double* coords, int64_t npts,
                            const DerivPlan& plan, void* out, bool out_f32, int64_t chunk, cudaStream_t s) {
    if (npts <= 0) return cudaSuccess;
    const int D = t.dim;
    if (D > 3) return cudaErrorInvalidValue;  // D = 4 evaluates with the direct kernel
    const int64_t cap = std::min<int64_t>(chunk, npts);
    const int64_t nb = g.nbuckets;
    // scratch: counts, cursor [nb], offsets [nb+1], records [cap] x (8 + 4D) bytes
    const size_t b_cnt = static_cast<size_t>(nb) * 4, b_off = static_cast<size_t>(nb + 1) * 4;
    auto up = [](size_t v) { return (v + 255) & ~size_t(255); };
    const size_t total = up(b_cnt) * 2 + up(b_off) + up(static_cast<size_t>(cap) * 4) * 2 +
                         up(static_cast<size_t>(cap) * 4 * D);
    void* mem = nullptr;
    cudaError_t e = cudaMallocAsync(&mem, total, s);
    if (e != cudaSuccess) return e;
    unsigned char* p = static_cast<unsigned char*>(mem);
    uint32_t* counts = reinterpret_cast<uint32_t*>(p);
    p += up(b_cnt);
    uint32_t* cursor = reinterpret_cast<uint32_t*>(p);
    p += up(b_cnt);
    uint32_t* offsets = reinterpret_cast<uint32_t*>(p);
    p += up(b_off);
    uint32_t* ridx = reinterpret_cast<uint32_t*>(p);
    p += up(static_cast<size_t>(cap) * 4);
    uint32_t* rcell = reinterpret_cast<uint32_t*>(p);
    p += up(static_cast<size_t>(cap) * 4);
    float* ru = reinterpret_cast<float*>(p);
    const int K = plan.k;
    const size_t ob = out_f32 ? 4 : 8;
    const int grid_eval = sm_count() * 6;
    for (int64_t p0 = 0; p0 < npts && e == cudaSuccess; p0 += cap) {
        const int64_t n = std::min(cap, npts - p0);
        const double* c = coords + p0 * D;
        switch (D) {
            case 1: e = launch_hist_scatter<1>(t, g, c, n, counts, offsets, cursor, ridx, rcell, ru, cap, s); break;
            case 2: e = launch_hist_scatter<2>(t, g, c, n, counts, offsets, cursor, ridx, rcell, ru, cap, s); break;
            case 3: e = launch_hist_scatter<3>(t, g, c, n, counts, offsets, cursor, ridx, rcell, ru, cap, s); break;
            default: e = cudaErrorInvalidValue;
        }
        if (e != cudaSuccess) break;
        void* o = static_cast<unsigned char*>(out) + static_cast<size_t>(p0) * K * ob;
        e = D <= 2 ? launch_bin_eval_d12(t, g, offsets, ridx, rcell, ru, cap, n, plan, o, out_f32, grid_eval, s)
                   : launch_bin_eval_d3(t, g, offsets, ridx, rcell, ru, cap, n, plan, o, out_f32, grid_eval, s);
    }
    cudaError_t e2 = cudaFreeAsync(mem, s);
    return e != cudaSuccess ? e : e2;
}

}  // namespace intp_gb300
