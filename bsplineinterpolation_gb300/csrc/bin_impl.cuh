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
//            written as one record {u_0 .. u_{D-1}, packed local span, index}
//            of D + 2 words to its pair's next slot
//   eval:    CTA j takes the j-th equal slice of the sorted records, stages the
//            tile of each bucket it meets, evaluates, writes out[index]
//
// Count and scatter aggregate their shared-memory atomics per warp
// (__match_any_sync): lanes of a warp that fall into one bucket take
// consecutive slots with a single atomic, so clustered queries neither
// serialise on a counter nor scatter their records.
//
// Queries are processed in chunks of the input. A chunk is large (millions of
// queries) so each bucket's tile is staged a few times per chunk only; its
// output writes land in a region small enough to stay in L2 until its
// sectors are complete.
#pragma once

#include <cstdint>

#include "basis32.cuh"
#include "device_common.cuh"
#include "launch.hpp"
#include "mixed_point.cuh"

namespace intp_gb300 {
namespace bin_detail {

constexpr int kBinThreads = 256;   // evaluation CTA
constexpr int kSortThreads = 512;  // count / scatter CTA

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

// Words per query record: u_0 .. u_{D-1}, packed local span, query index.
template <int D>
__host__ __device__ constexpr int rec_words() {
    return D + 2;
}

// Counting sort without global atomics. CTA `blk` owns the input slice
// [blk*S, (blk+1)*S); count_kernel writes its per-bucket counts to
// blkcount[b * nblk + blk] (bucket-major), an exclusive scan over that array
// gives every (bucket, CTA) pair its first slot, and scatter_kernel re-reads
// the same slice and places each query at its pair's cursor (shared-memory
// atomics only). The first slot of bucket b is then scan[b * nblk]. Every
// thread runs the same number of loop trips so the warp-wide match sees all
// lanes.

template <int D>
__global__ void __launch_bounds__(kSortThreads) count_kernel(TableDev t, BinGeom g, const double* __restrict__ coords,
                                                            int64_t n, int64_t slice, uint32_t* __restrict__ blkcount) {
    extern __shared__ uint32_t sh_count[];
    const int nblk = gridDim.x, blk = blockIdx.x;
    for (int64_t b = threadIdx.x; b < g.nbuckets; b += blockDim.x) sh_count[b] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t p0 = blk * slice, p1 = (p0 + slice < n) ? p0 + slice : n;
    for (int64_t base = p0; base < p1; base += blockDim.x) {
        const int64_t p = base + threadIdx.x;
        const bool valid = p < p1;
        uint32_t b = 0xFFFFFFFFu;
        if (valid) {
            int64_t cl[D];
#pragma unroll
            for (int d = 0; d < D; ++d) cl[d] = span_only(t.ax[d], t.order, __ldg(coords + p * D + d)) - t.order;
            b = bucket_of<D>(g, cl);
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, b);
        if (valid && lane == __ffs(peers) - 1) atomicAdd(&sh_count[b], static_cast<uint32_t>(__popc(peers)));
    }
    __syncthreads();
    for (int64_t b = threadIdx.x; b < g.nbuckets; b += blockDim.x) blkcount[b * nblk + blk] = sh_count[b];
}

template <int D>
__global__ void __launch_bounds__(kSortThreads) scatter_kernel(TableDev t, BinGeom g, const double* __restrict__ coords,
                                                              int64_t n, int64_t slice,
                                                              const uint32_t* __restrict__ blkoffset,
                                                              uint32_t* __restrict__ rec) {
    extern __shared__ uint32_t sh_cursor[];
    const int nblk = gridDim.x, blk = blockIdx.x;
    for (int64_t b = threadIdx.x; b < g.nbuckets; b += blockDim.x) sh_cursor[b] = blkoffset[b * nblk + blk];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const int64_t p0 = blk * slice, p1 = (p0 + slice < n) ? p0 + slice : n;
    for (int64_t base = p0; base < p1; base += blockDim.x) {
        const int64_t p = base + threadIdx.x;
        const bool valid = p < p1;
        uint32_t b = 0xFFFFFFFFu, packed = 0;
        float u[D];
        if (valid) {
            int64_t cl[D];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                cl[d] = span_and_offset(t.ax[d], t.order, __ldg(coords + p * D + d), u[d]) - t.order;
                packed |= static_cast<uint32_t>(cl[d] & ((1LL << g.lb[d]) - 1)) << g.shift[d];
            }
            b = bucket_of<D>(g, cl);
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, b);
        const int leader = __ffs(peers) - 1;
        uint32_t first = 0;
        if (valid && lane == leader) first = atomicAdd(&sh_cursor[b], static_cast<uint32_t>(__popc(peers)));
        first = __shfl_sync(0xFFFFFFFFu, first, leader);
        if (valid) {
            const uint32_t slot = first + static_cast<uint32_t>(__popc(peers & lt_mask));
            uint32_t* r = rec + static_cast<int64_t>(slot) * rec_words<D>();
#pragma unroll
            for (int d = 0; d < D; ++d) r[d] = __float_as_uint(u[d]);
            r[D] = packed;
            r[D + 1] = static_cast<uint32_t>(p);
        }
    }
}

constexpr int ipow_c(int b, int e) { return e == 0 ? 1 : b * ipow_c(b, e - 1); }

// Compile-time tile shape: P_d = 2^bucket_log2 + O per axis, row-major.
template <int D, int O>
struct TileShape {
    static constexpr int P(int d) { return (1 << bucket_log2(D, d)) + O; }
    static constexpr int S(int d) { return d >= D - 1 ? 1 : P(d + 1) * S(d + 1); }
    static constexpr int elems() { return P(0) * S(0); }
    static constexpr int rows() { return elems() / P(D - 1); }
};

// Control-point index along axis a of tile position org + i (periodic wrap,
// clamp at the end of a non-periodic axis: positions past the last control
// point are never read by a query of the bucket).
__device__ __forceinline__ int64_t tile_index(const AxisDev& a, int64_t gi) {
    return a.periodic ? gi % a.n : (gi < a.n ? gi : a.n - 1);
}

template <int D, int O>
__global__ void __launch_bounds__(kBinThreads, 2) eval_kernel(TableDev t, BinGeom g, const uint32_t* __restrict__ blkoffset,
                                                           int nblk, const uint32_t* __restrict__ rec, int64_t nrec,
                                                           DerivPlan plan, void* __restrict__ out, int out_f32) {
    using TS = TileShape<D, O>;
    constexpr int RW = rec_words<D>();
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
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int PL = TS::P(D - 1);  // tile row length (last axis)
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
            for (int d = 0; d < D; ++d) off += tile_index(t.ax[d], org[d] + TS::P(d) / 2) * t.ax[d].stride;
            sh_cref = __ldg(cp + off);
        }
        __syncthreads();
        const float cref = sh_cref;
        // one warp per tile row (contiguous along the last axis)
        for (int row = warp; row < TS::rows(); row += kBinThreads / 32) {
            int64_t off = 0;
            int rem = row;
#pragma unroll
            for (int d = D - 2; d >= 0; --d) {
                const int i = rem % TS::P(d);
                rem /= TS::P(d);
                off += tile_index(t.ax[d], org[d] + i) * t.ax[d].stride;
            }
            const AxisDev& al = t.ax[D - 1];
            for (int i = lane; i < PL; i += 32)
                tile[row * PL + i] = __ldg(cp + off + tile_index(al, org[D - 1] + i)) - cref;
        }
        __syncthreads();
        // records are software-pipelined: the next one loads while the
        // current one is evaluated
        uint32_t nx[RW];
        int64_t rr = r + threadIdx.x;
        if (rr < end) {
#pragma unroll
            for (int j = 0; j < RW; ++j) nx[j] = __ldg(rec + rr * RW + j);
        }
        for (; rr < end; rr += blockDim.x) {
            uint32_t cur[RW];
#pragma unroll
            for (int j = 0; j < RW; ++j) cur[j] = nx[j];
            const int64_t nr = rr + blockDim.x;
            if (nr < end) {
#pragma unroll
                for (int j = 0; j < RW; ++j) nx[j] = __ldg(rec + nr * RW + j);
            }
            float u[D];
            int64_t c[D];
            float base[D][W];
            int tb = 0;
            const uint32_t packed = cur[D];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                u[d] = __uint_as_float(cur[d]);
                const int cl = static_cast<int>((packed >> g.shift[d]) & ((1u << bucket_log2(D, d)) - 1u));
                c[d] = org[d] + cl + O;
                tb += cl * TS::S(d);
                axis_weights32<O>(t.ax[d], c[d], u[d], 0, base[d]);
            }
            const float* tl = tile + tb;
            const int64_t o0 = static_cast<int64_t>(cur[D + 1]) * K;
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
