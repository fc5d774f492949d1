// Host side of the binned evaluation: bucket geometry, chunk loop, launches
// of the histogram / scan / scatter kernels (the evaluation kernels are
// instantiated in bin_eval_d12.cu and bin_eval_d34.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "bin_impl.cuh"

namespace intp_gb300 {

namespace bin_detail {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* sh, uint32_t& total) {
    const int tid = threadIdx.x;
    sh[tid] = v;
    __syncthreads();
    for (int off = 1; off < kScanThreads; off <<= 1) {
        const uint32_t a = tid >= off ? sh[tid - off] : 0u;
        __syncthreads();
        sh[tid] += a;
        __syncthreads();
    }
    total = sh[kScanThreads - 1];
    const uint32_t r = sh[tid] - v;
    __syncthreads();
    return r;
}

// per-tile sums of x[0..n)
__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const uint32_t* __restrict__ x, int64_t n,
                                                                   uint32_t* __restrict__ tile_sum) {
    __shared__ uint32_t sh[kScanThreads];
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) s += x[base + k];
    uint32_t total;
    block_exclusive_scan(s, sh, total);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// exclusive scan of the tile sums in place (one block; ntiles <= 4096)
__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(uint32_t* __restrict__ tile_sum, int64_t ntiles) {
    __shared__ uint32_t sh[kScanThreads];
    const int64_t base = threadIdx.x * kScanItems;
    uint32_t v[kScanItems], s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < ntiles ? tile_sum[base + k] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan(s, sh, total);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < ntiles) {
            tile_sum[base + k] = run;
            run += v[k];
        }
}

// exclusive scan of x into y, each tile offset by its scanned tile sum
__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const uint32_t* __restrict__ x, int64_t n,
                                                                  const uint32_t* __restrict__ tile_sum,
                                                                  uint32_t* __restrict__ y) {
    __shared__ uint32_t sh[kScanThreads];
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems], s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? x[base + k] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan(s, sh, total) + tile_sum[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) {
            y[base + k] = run;
            run += v[k];
        }
}

// Knot spans of the queries in input order, decoded from the records the
// locate kernel wrote: the bucket in the tag's high bits, the span within the
// bucket in its low kCellBits bits (the inverse of locate_kernel's packing).
template <int D>
__global__ void decode_spans_kernel(BinGeom g, int order, const uint32_t* __restrict__ in_rec, int64_t n,
                                    int64_t* __restrict__ cells) {
    constexpr int RW = rec_words<D>();
    for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < n;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        uint32_t w[RW];
        rec_load<D>(in_rec, p, w);
        const uint32_t tag = w[RW - 1];
        uint32_t b = tag >> kCellBits;
#pragma unroll
        for (int d = D - 1; d >= 0; --d) {
            const uint32_t bc = b % static_cast<uint32_t>(g.nb[d]);
            b /= static_cast<uint32_t>(g.nb[d]);
            const uint32_t local = (tag >> g.shift[d]) & ((1u << g.lb[d]) - 1u);
            cells[p * D + d] = static_cast<int64_t>((bc << g.lb[d]) | local) + order;
        }
    }
}

}  // namespace bin_detail

namespace {

constexpr int32_t kSmemBucketLimit = 48 * 1024;

int sort_ctas_per_sm() {
    static int v = 0;
    if (v == 0) {
        const char* e = std::getenv("INTP_GB300_SORT_CTAS_PER_SM");
        v = e ? std::atoi(e) : 2;
        if (v < 1 || v > 3) v = 2;
    }
    return v;
}

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
cudaError_t launch_sort(const TableDev& t, const BinGeom& g, const double* coords, int64_t n, int nblk,
                        uint32_t* blkcount, uint32_t* blkoffset, uint32_t* tile_sum, uint32_t* rec, int64_t slice,
                        cudaStream_t s) {
    using namespace bin_detail;
    const size_t smem = static_cast<size_t>(g.nbuckets) * 4;
    auto kc = count_kernel<D>;
    auto ks = scatter_kernel<D>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kc, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(ks, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    kc<<<nblk, kLocateThreads, smem, s>>>(t, g, coords, n, slice, blkcount);
    note_launch();
    const int64_t m = g.nbuckets * nblk;
    const int64_t ntiles = (m + kScanTile - 1) / kScanTile;
    scan_reduce_kernel<<<static_cast<int>(ntiles), kScanThreads, 0, s>>>(blkcount, m, tile_sum);
    note_launch();
    scan_tiles_kernel<<<1, kScanThreads, 0, s>>>(tile_sum, ntiles);
    note_launch();
    scan_apply_kernel<<<static_cast<int>(ntiles), kScanThreads, 0, s>>>(blkcount, m, tile_sum, blkoffset);
    note_launch();
    ks<<<nblk, kSortThreads, smem, s>>>(t, g, coords, n, slice, blkoffset, rec);
    note_launch();
    return cudaGetLastError();
}

}  // namespace

template <int D>
cudaError_t launch_span_readout(const TableDev& t, const BinGeom& g, const double* coords, int64_t n, int nblk,
                                uint32_t* blkcount, uint32_t* in_rec, int64_t* cells, cudaStream_t s) {
    using namespace bin_detail;
    const size_t smem = static_cast<size_t>(g.nbuckets) * 4;
    auto kl = locate_kernel<D>;
    if (smem > 48 * 1024) {
        const cudaError_t e =
            cudaFuncSetAttribute(kl, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    const int64_t slice = (n + nblk - 1) / nblk;
    kl<<<nblk, kLocateThreads, smem, s>>>(t, g, coords, n, slice, in_rec, blkcount);
    note_launch();
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, int64_t{sm_count()} * 8);
    decode_spans_kernel<D><<<static_cast<int>(blocks), 256, 0, s>>>(g, t.order, in_rec, n, cells);
    note_launch();
    return cudaGetLastError();
}

int bin_record_words(int dim) { return dim == 1 ? bin_detail::rec_words<1>() : bin_detail::rec_words<2>(); }

cudaError_t bin_sort_chunk(const TableDev& t, const BinGeom& g, const double* coords, int64_t n, int nblk,
                           uint32_t* blkcount, uint32_t* blkoffset, uint32_t* tile_sum, uint32_t* rec, int64_t* slice,
                           cudaStream_t s) {
    if (nblk < 1 || nblk > bin_detail::kMaxSortBlocks) return cudaErrorInvalidValue;
    const int64_t sl = (n + nblk - 1) / nblk;
    if (sl >= bin_detail::kMaxSlice) return cudaErrorInvalidValue;
    *slice = sl;
    switch (t.dim) {
        case 1: return launch_sort<1>(t, g, coords, n, nblk, blkcount, blkoffset, tile_sum, rec, sl, s);
        case 2: return launch_sort<2>(t, g, coords, n, nblk, blkcount, blkoffset, tile_sum, rec, sl, s);
        case 3: return launch_sort<3>(t, g, coords, n, nblk, blkcount, blkoffset, tile_sum, rec, sl, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t binned_span_readout(const TableDev& t, const BinGeom& g, const double* coords, int64_t npts,
                                int64_t* cells, cudaStream_t s) {
    if (npts <= 0) return cudaSuccess;
    const int D = t.dim;
    if (D > 3) return cudaErrorInvalidValue;
    const int nblk = sm_count();
    // the production chunk bound: a sort CTA's slice stays below kMaxSlice
    const int64_t cap = std::min<int64_t>(npts, int64_t{nblk} * (bin_detail::kMaxSlice - 1));
    auto up = [](size_t v) { return (v + 255) & ~size_t(255); };
    const size_t b_m = up(static_cast<size_t>(g.nbuckets * nblk) * 4);
    const size_t total = b_m + up(static_cast<size_t>(cap) * 4 * bin_record_words(D));
    void* mem = nullptr;
    cudaError_t e = cudaMallocAsync(&mem, total, s);
    if (e != cudaSuccess) return e;
    uint32_t* blkcount = static_cast<uint32_t*>(mem);
    uint32_t* in_rec = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(mem) + b_m);
    for (int64_t p0 = 0; p0 < npts && e == cudaSuccess; p0 += cap) {
        const int64_t n = std::min(cap, npts - p0);
        const double* c = coords + p0 * D;
        int64_t* o = cells + p0 * D;
        switch (D) {
            case 1: e = launch_span_readout<1>(t, g, c, n, nblk, blkcount, in_rec, o, s); break;
            case 2: e = launch_span_readout<2>(t, g, c, n, nblk, blkcount, in_rec, o, s); break;
            default: e = launch_span_readout<3>(t, g, c, n, nblk, blkcount, in_rec, o, s); break;
        }
    }
    const cudaError_t e2 = cudaFreeAsync(mem, s);
    return e != cudaSuccess ? e : e2;
}

BinGeom make_bin_geom(const TableDev& t) {
    BinGeom g{};
    const int D = t.dim, O = t.order;
    g.dim = D;
    int shift = 0;
    g.nbuckets = 1;
    int32_t stride = 1;
    for (int d = D - 1; d >= 0; --d) {
        const int lb = bucket_log2(D, d);
        g.lb[d] = lb;
        g.P[d] = (1 << lb) + O;
        g.nb[d] = static_cast<int32_t>((t.ax[d].ncells + (int64_t{1} << lb) - 1) >> lb);
        g.tstride[d] = stride;
        // rows of the last axis are padded to a multiple of 4 floats
        stride *= d == D - 1 ? ((g.P[d] + 3) & ~3) : g.P[d];
    }
    // the span within the bucket packs row-major, the last axis in the low
    // bits: ordering records by it orders them as the tile lies in memory
    for (int d = D - 1; d >= 0; --d) {
        g.shift[d] = shift;
        shift += g.lb[d];
        g.nbuckets *= g.nb[d];
    }
    g.tile_elems = stride;
    // the binned kernels index spans with 32 bits and keep the bucket in the
    // 20 high bits of a record's tag word
    bool small = g.nbuckets <= kSmemBucketLimit;
    for (int d = 0; d < D; ++d) small = small && t.ax[d].nknots < (int64_t{1} << 30);
    g.smem_buckets = small ? static_cast<int32_t>(g.nbuckets) : 0;
    return g;
}

cudaError_t run_binned_eval(const TableDev& t, const BinGeom& g, const CUtensorMap* tmap, const double* coords,
                            int64_t npts, const DerivPlan& plan, void* out, bool out_f32, int64_t chunk,
                            cudaStream_t s) {
    if (npts <= 0) return cudaSuccess;
    const int D = t.dim;
    if (D > 3) return cudaErrorInvalidValue;  // D = 4 evaluates with the direct kernel
    // count CTAs per SM (INTP_GB300_SORT_CTAS_PER_SM, 1..3; default 2):
    // fewer slices mean fewer (bucket, slice) segments that the scatter
    // fills at once, more of them a better spread of the count work
    const int nblk = sm_count() * sort_ctas_per_sm();
    // a record names its query by its index within a sort CTA's slice
    // (below kMaxSlice)
    const int64_t cap = std::min<int64_t>(std::min<int64_t>(chunk, npts), int64_t{nblk} * (bin_detail::kMaxSlice - 1));
    const int64_t m = g.nbuckets * nblk;
    const int64_t ntiles = (m + bin_detail::kScanTile - 1) / bin_detail::kScanTile;
    if (ntiles > bin_detail::kScanThreads * bin_detail::kScanItems) return cudaErrorInvalidValue;
    auto up = [](size_t v) { return (v + 255) & ~size_t(255); };
    const size_t b_m = up(static_cast<size_t>(m) * 4), b_t = up(static_cast<size_t>(ntiles) * 4);
    const size_t b_r = up(static_cast<size_t>(cap) * 4 * bin_record_words(D));
    const size_t total = b_m * 2 + b_t + b_r;
    void* mem = nullptr;
    cudaError_t e = cudaMallocAsync(&mem, total, s);
    if (e != cudaSuccess) return e;
    unsigned char* p = static_cast<unsigned char*>(mem);
    uint32_t* blkcount = reinterpret_cast<uint32_t*>(p);
    p += b_m;
    uint32_t* blkoffset = reinterpret_cast<uint32_t*>(p);
    p += b_m;
    uint32_t* tile_sum = reinterpret_cast<uint32_t*>(p);
    p += b_t;
    uint32_t* rec = reinterpret_cast<uint32_t*>(p);
    const int K = plan.k * (t.channels > 1 ? t.channels : 1);  // output values per query
    const size_t ob = out_f32 ? 4 : 8;
    const int grid_eval = sm_count();  // the launchers fill each SM
    for (int64_t p0 = 0; p0 < npts && e == cudaSuccess; p0 += cap) {
        const int64_t n = std::min(cap, npts - p0);
        const double* c = coords + p0 * D;
        int64_t slice = 0;
        e = bin_sort_chunk(t, g, c, n, nblk, blkcount, blkoffset, tile_sum, rec, &slice, s);
        if (e != cudaSuccess) break;
        void* o = static_cast<unsigned char*>(out) + static_cast<size_t>(p0) * K * ob;
        e = D <= 2 ? launch_bin_eval_d12(t, g, tmap, blkoffset, nblk, slice, rec, n, plan, o, out_f32, grid_eval, s)
                   : launch_bin_eval_d3(t, g, tmap, blkoffset, nblk, slice, rec, n, plan, o, out_f32, grid_eval, s);
    }
    cudaError_t e2 = cudaFreeAsync(mem, s);
    return e != cudaSuccess ? e : e2;
}

}  // namespace intp_gb300
