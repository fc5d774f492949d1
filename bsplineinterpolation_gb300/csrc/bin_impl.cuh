// Binned evaluation (mixed form): queries are counting-sorted by spatial
// bucket, then every bucket is evaluated against a shared-memory tile of the
// control points it touches.
//
// Random queries gathered straight from a 256^3 table touch ~22 sectors each
// and run at L1/L2 gather speed; after binning, the (O+1)^D neighbourhood of
// every query of a bucket comes from one tile of prod(B_d + O) control points
// staged once in shared memory.
//
//   count:   bucket of every query -> per-(bucket, CTA) counts
//   scan:    exclusive prefix sum over (bucket, CTA) -> first slot of each pair
//   scatter: exact span (integer keys) and FP32 local offsets of every query,
//            written as a compact record {index, packed local span, u_d} to its
//            pair's slots (shared-memory cursors; no global atomics)
//   eval:    CTA j takes the j-th equal slice of the sorted records, stages the
//            tile of each bucket it meets, evaluates, writes out[index]
//
// Queries are processed in chunks of the input so each chunk's scattered
// output writes stay resident in L2 until their sectors are complete.
#pragma once

#include <cstdint>

#include "basis32.cuh"
#include "device_common.cuh"
#include "launch.hpp"
#include "mixed_point.cuh"

namespace intp_gb300 {
namespace bin_detail {

constexpr int kBinThreads = 256;    // evaluation CTA
constexpr int kSortThreads = 1024;  // count / scatter CTA

// Exact span and FP32 local offset of one coordinate on axis a (mixed form).
__device__ __forceinline__ int64_t span_and_offset(const AxisDev& a, int order, double x, float& u) {
    if (a.periodic) x = periodic_wrap(a, x);
    const int64_t h = a.uniform ? uniform_hint(a, x) : static_cast<int64_t>(order);
    const int64_t c = locate_span(a, order, knot_key(x), h);
    float xh, xl;
    split_double(x, xh, xl);
    u = (xh - __ldg(a.khi + c)) + (xl - __ldg(a.klo + c));
    return c;
}

__device__ __forceinline__ int64_t span_only(const AxisDev& a, int order, double x) {
    if (a.periodic) x = periodic_wrap(a, x);
    const int64_t h = a.uniform ? uniform_hint(a, x) : static_cast<int64_t>(order);
    return locate_span(a, order, knot_key(x), h);
}

template <int D>
__device__ __forceinline__ uint32_t bucket_of(const BinGeom& g, const int64_t (&cl)[D]) {
    uint32_t b = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) b = b * static_cast<uint32_t>(g.nb[d]) + static_cast<uint32_t>(cl[d] >> g.lb[d]);
    return b;
}

// Counting sort without global atomics. CTA `blk` owns the input slice
// [blk*S, (blk+1)*S); count_kernel writes its per-bucket counts to
// blkcount[b * nblk + blk] (bucket-major), an exclusive scan over that array
// gives every (bucket, CTA) pair its first slot, and scatter_kernel re-reads
// the same slice and places each query at its pair's cursor (shared-memory
// atomics only). The first slot of bucket b is then scan[b * nblk].

template <int D>
__global__ void __launch_bounds__(kSortThreads) count_kernel(TableDev t, BinGeom g, const double* __restrict__ coords,
                                                            int64_t n, int64_t slice, uint32_t* __restrict__ blkcount) {
    extern __shared__ uint32_t sh_count[];
    const int nblk = gridDim.x, blk = blockIdx.x;
    for (int64_t b = threadIdx.x; b < g.nbuckets; b += blockDim.x) sh_count[b] = 0;
    __syncthreads();
    const int64_t p0 = blk * slice, p1 = (p0 + slice < n) ? p0 + slice : n;
    for (int64_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        int64_t cl[D];
#pragma unroll
        for (int d = 0; d < D; ++d) cl[d] = span_only(t.ax[d], t.order, __ldg(coords + p * D + d)) - t.order;
        atomicAdd(&sh_count[bucket_of<D>(g, cl)], 1u);
    }
    __syncthreads();
    for (int64_t b = threadIdx.x; b < g.nbuckets; b += blockDim.x) blkcount[b * nblk + blk] = sh_count[b];
}

template <int D>
__global__ void __launch_bounds__(kSortThreads) scatter_kernel(TableDev t, BinGeom g, const double* __restrict__ coords,
                                                              int64_t n, int64_t slice,
                                                              const uint32_t* __restrict__ blkoffset,
                                                              uint32_t* __restrict__ ridx, uint32_t* __restrict__ rcell,
                                                              float* __restrict__ ru, int64_t cap) {
    extern __shared__ uint32_t sh_cursor[];
    const int nblk = gridDim.x, blk = blockIdx.x;
    for (int64_t b = threadIdx.x; b < g.nbuckets; b += blockDim.x) sh_cursor[b] = blkoffset[b * nblk + blk];
    __syncthreads();
    const int64_t p0 = blk * slice, p1 = (p0 + slice < n) ? p0 + slice : n;
    for (int64_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        int64_t cl[D];
        float u[D];
        uint32_t packed = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            cl[d] = span_and_offset(t.ax[d], t.order, __ldg(coords + p * D + d), u[d]) - t.order;
            packed |= static_cast<uint32_t>(cl[d] & ((1LL << g.lb[d]) - 1)) << g.shift[d];
        }
        const uint32_t slot = atomicAdd(&sh_cursor[bucket_of<D>(g, cl)], 1u);
        ridx[slot] = static_cast<uint32_t>(p);
        rcell[slot] = packed;
#pragma unroll
        for (int d = 0; d < D; ++d) ru[d * cap + slot] = u[d];
    }
}

constexpr int ipow_c(int b, int e) { return e == 0 ? 1 : b * ipow_c(b, e - 1); }

// Compile-time tile shape: P_d = 2^bucket_log2 + O per axis, row-major.
template <int D, int O>
struct TileShape {
    static constexpr int P(int d) { return (1 << bucket_log2(D, d)) + O; }
    static constexpr int S(int d) { return d >= D - 1 ? 1 : P(d + 1) * S(d + 1); }
    static constexpr int elems() { return P(0) * S(0); }
};

template <int D, int O>
__global__ void __launch_bounds__(kBinThreads, 2) eval_kernel(TableDev t, BinGeom g, const uint32_t* __restrict__ blkoffset,
                                                           int nblk, const uint32_t* __restrict__ ridx,
                                                           const uint32_t* __restrict__ rcell,
                                                           const float* __restrict__ ru, int64_t cap, int64_t nrec,
                                                           DerivPlan plan, void* __restrict__ out, int out_f32) {
    using TS = TileShape<D, O>;
    extern __shared__ float tile[];
    __shared__ float sh_cref;
    __shared__ DerivPlan sh_plan;  // indexed by runtime output / group numbers
    constexpr int W = O + 1;
    const float* __restrict__ cp = static_cast<const float*>(t.ctrl);
    const int K = plan.k;
    const int64_t r0 = nrec * blockIdx.x / gridDim.x, r1 = nrec * (blockIdx.x + 1) / gridDim.x;
    if (r0 >= r1) return;
    if (threadIdx.x == 0) sh_plan = plan;
    __syncthreads();
    // first slot of bucket b (bucket g.nbuckets: one past the last record)
    auto bstart = [&](int64_t bb) -> int64_t {
        return bb >= g.nbuckets ? nrec : static_cast<int64_t>(__ldg(blkoffset + bb * nblk));
    };
    int64_t lo = 0, hi = g.nbuckets;
    while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (bstart(mid) <= r0)
            lo = mid;
        else
            hi = mid;
    }
    int64_t b = lo;
    int64_t r = r0;
    while (r < r1) {
        while (bstart(b + 1) <= r) ++b;
        const int64_t bend = bstart(b + 1);
        const int64_t end = bend < r1 ? bend : r1;
        int64_t org[D];
        {
            int64_t rem = b;
#pragma unroll
            for (int d = D - 1; d >= 0; --d) {
                org[d] = (rem % g.nb[d]) << bucket_log2(D, d);
                rem /= g.nb[d];
            }
        }
        __syncthreads();
        // The tile is stored relative to a reference control point near its
        // centre: value weights sum to 1 and derivative weights to 0, so the
        // FP32 rounding of the weights only multiplies the local variation.
        if (threadIdx.x == 0) {
            int64_t off = 0;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const AxisDev& a = t.ax[d];
                int64_t gi = org[d] + TS::P(d) / 2;
                gi = a.periodic ? gi % a.n : (gi < a.n ? gi : a.n - 1);
                off += gi * a.stride;
            }
            sh_cref = __ldg(cp + off);
        }
        __syncthreads();
        const float cref = sh_cref;
        for (int e = threadIdx.x; e < TS::elems(); e += blockDim.x) {
            int64_t off = 0;
            int rem = e;
#pragma unroll
            for (int d = D - 1; d >= 0; --d) {
                const int i = rem % TS::P(d);
                rem /= TS::P(d);
                const AxisDev& a = t.ax[d];
                int64_t gi = org[d] + i;
                gi = a.periodic ? gi % a.n : (gi < a.n ? gi : a.n - 1);
                off += gi * a.stride;
            }
            tile[e] = __ldg(cp + off) - cref;
        }
        __syncthreads();
        // records are software-pipelined: the next one loads while the
        // current one is evaluated
        uint32_t n_idx = 0, n_packed = 0;
        float n_u[D];
        int64_t rr = r + threadIdx.x;
        if (rr < end) {
            n_idx = __ldg(ridx + rr);
            n_packed = __ldg(rcell + rr);
#pragma unroll
            for (int d = 0; d < D; ++d) n_u[d] = __ldg(ru + d * cap + rr);
        }
        for (; rr < end; rr += blockDim.x) {
            const uint32_t idx = n_idx;
            const uint32_t packed = n_packed;
            float u[D];
#pragma unroll
            for (int d = 0; d < D; ++d) u[d] = n_u[d];
            const int64_t nx = rr + blockDim.x;
            if (nx < end) {
                n_idx = __ldg(ridx + nx);
                n_packed = __ldg(rcell + nx);
#pragma unroll
                for (int d = 0; d < D; ++d) n_u[d] = __ldg(ru + d * cap + nx);
            }
            int64_t c[D];
            float base[D][W];
            int tb = 0;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const int cl = static_cast<int>((packed >> g.shift[d]) & ((1u << bucket_log2(D, d)) - 1u));
                c[d] = org[d] + cl + O;
                tb += cl * TS::S(d);
                axis_weights32<O>(t.ax[d], c[d], u[d], 0, base[d]);
            }
            const float* tl = tile + tb;
            const int64_t o0 = static_cast<int64_t>(idx) * K;
            mixed_point_outputs<D, O>(
                t, sh_plan, c, u, base, cref,
                [tl](const int (&ix)[D]) {
                    int off = 0;
#pragma unroll
                    for (int d = 0; d < D; ++d) off += ix[d] * TS::S(d);
                    return tl[off];
                },
                [out, out_f32, o0](int k, float v) {
                    if (out_f32)
                        static_cast<float*>(out)[o0 + k] = v;
                    else
                        static_cast<double*>(out)[o0 + k] = static_cast<double>(v);
                });
        }
        r = end;
    }
}

}  // namespace bin_detail
}  // namespace intp_gb300
