// Binned evaluation (mixed form): queries are counting-sorted by spatial
// bucket, then every bucket is evaluated against a shared-memory tile of the
// control points it touches.
//
// Random queries gathered straight from a 256^3 table touch ~22 sectors each
// and run at L1/L2 gather speed; after binning, the (O+1)^D neighbourhood of
// every query of a bucket comes from one tile of prod(B_d + O) control points
// staged once in shared memory.
//
//   hist:    bucket of every query -> per-bucket counts (CTA-local histogram,
//            one global atomic per touched bucket and CTA)
//   scan:    exclusive prefix sum -> bucket offsets, scatter cursors
//   scatter: exact span (integer keys) and FP32 local offsets of every query,
//            written as a compact record {index, packed local span, u_d} to the
//            bucket's slot range (CTA-aggregated atomics)
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

namespace intp_gb300 {
namespace bin_detail {

constexpr int kBinThreads = 256;
constexpr int kScatterItems = 4;  // queries per thread per scatter round

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

template <int D>
__global__ void __launch_bounds__(kBinThreads) hist_kernel(TableDev t, BinGeom g, const double* __restrict__ coords,
                                                           int64_t n, uint32_t* __restrict__ counts) {
    extern __shared__ uint32_t sh_count[];
    const bool local = g.nbuckets <= g.smem_buckets;
    if (local) {
        for (int64_t b = threadIdx.x; b < g.nbuckets; b += blockDim.x) sh_count[b] = 0;
        __syncthreads();
    }
    for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < n;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t cl[D];
#pragma unroll
        for (int d = 0; d < D; ++d) cl[d] = span_only(t.ax[d], t.order, __ldg(coords + p * D + d)) - t.order;
        const uint32_t b = bucket_of<D>(g, cl);
        if (local)
            atomicAdd(&sh_count[b], 1u);
        else
            atomicAdd(&counts[b], 1u);
    }
    if (local) {
        __syncthreads();
        for (int64_t b = threadIdx.x; b < g.nbuckets; b += blockDim.x)
            if (sh_count[b]) atomicAdd(&counts[b], sh_count[b]);
    }
}

template <int D>
__global__ void __launch_bounds__(kBinThreads) scatter_kernel(TableDev t, BinGeom g, const double* __restrict__ coords,
                                                              int64_t n, uint32_t* __restrict__ cursor,
                                                              uint32_t* __restrict__ ridx, uint32_t* __restrict__ rcell,
                                                              float* __restrict__ ru, int64_t cap) {
    extern __shared__ uint32_t sh[];
    uint32_t* sh_count = sh;
    uint32_t* sh_base = sh + g.smem_buckets;
    const bool local = g.nbuckets <= g.smem_buckets;
    if (local) {
        for (int64_t b = threadIdx.x; b < g.nbuckets; b += blockDim.x) sh_count[b] = 0;
        __syncthreads();
    }
    const int64_t per_round = static_cast<int64_t>(blockDim.x) * kScatterItems;
    for (int64_t base = blockIdx.x * per_round; base < n; base += static_cast<int64_t>(gridDim.x) * per_round) {
        uint32_t bkt[kScatterItems], rank[kScatterItems], packed[kScatterItems];
        float u[kScatterItems][D];
        bool valid[kScatterItems];
#pragma unroll
        for (int it = 0; it < kScatterItems; ++it) {
            const int64_t p = base + it * blockDim.x + threadIdx.x;
            valid[it] = p < n;
            bkt[it] = 0;
            packed[it] = 0;
            if (valid[it]) {
                int64_t cl[D];
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    cl[d] = span_and_offset(t.ax[d], t.order, __ldg(coords + p * D + d), u[it][d]) - t.order;
                    packed[it] |= static_cast<uint32_t>(cl[d] & ((1LL << g.lb[d]) - 1)) << g.shift[d];
                }
                bkt[it] = bucket_of<D>(g, cl);
                if (local)
                    rank[it] = atomicAdd(&sh_count[bkt[it]], 1u);
                else
                    rank[it] = atomicAdd(&cursor[bkt[it]], 1u);
            }
        }
        if (local) {
            __syncthreads();
            // the query that took rank 0 reserves its bucket's slot range
#pragma unroll
            for (int it = 0; it < kScatterItems; ++it)
                if (valid[it] && rank[it] == 0) sh_base[bkt[it]] = atomicAdd(&cursor[bkt[it]], sh_count[bkt[it]]);
            __syncthreads();
        }
#pragma unroll
        for (int it = 0; it < kScatterItems; ++it) {
            if (!valid[it]) continue;
            const int64_t p = base + it * blockDim.x + threadIdx.x;
            const uint32_t slot = local ? sh_base[bkt[it]] + rank[it] : rank[it];
            ridx[slot] = static_cast<uint32_t>(p);
            rcell[slot] = packed[it];
#pragma unroll
            for (int d = 0; d < D; ++d) ru[d * cap + slot] = u[it][d];
        }
        if (local) {
            __syncthreads();
#pragma unroll
            for (int it = 0; it < kScatterItems; ++it)
                if (valid[it] && rank[it] == 0) sh_count[bkt[it]] = 0;
            __syncthreads();
        }
    }
}

constexpr int ipow_c(int b, int e) { return e == 0 ? 1 : b * ipow_c(b, e - 1); }

template <int D, int O>
__global__ void __launch_bounds__(kBinThreads) eval_kernel(TableDev t, BinGeom g, const uint32_t* __restrict__ offsets,
                                                           const uint32_t* __restrict__ ridx,
                                                           const uint32_t* __restrict__ rcell,
                                                           const float* __restrict__ ru, int64_t cap, int64_t nrec,
                                                           DerivPlan plan, void* __restrict__ out, int out_f32) {
    extern __shared__ float tile[];
    constexpr int W = O + 1;
    constexpr int ROWS = ipow_c(W, D - 1);
    const float* __restrict__ cp = static_cast<const float*>(t.ctrl);
    const int K = plan.k;
    const int64_t r0 = nrec * blockIdx.x / gridDim.x, r1 = nrec * (blockIdx.x + 1) / gridDim.x;
    if (r0 >= r1) return;
    // bucket holding record r0: last b with offsets[b] <= r0
    int64_t lo = 0, hi = g.nbuckets;
    while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (offsets[mid] <= static_cast<uint32_t>(r0))
            lo = mid;
        else
            hi = mid;
    }
    int64_t b = lo;
    int64_t r = r0;
    while (r < r1) {
        while (offsets[b + 1] <= static_cast<uint32_t>(r)) ++b;
        const int64_t end = offsets[b + 1] < static_cast<uint32_t>(r1) ? offsets[b + 1] : r1;
        // bucket origin (first local span) per axis
        int64_t org[D];
        {
            int64_t rem = b;
#pragma unroll
            for (int d = D - 1; d >= 0; --d) {
                org[d] = (rem % g.nb[d]) << g.lb[d];
                rem /= g.nb[d];
            }
        }
        __syncthreads();
        // stage the tile: control points org_d .. org_d + B_d + O - 1 per axis
        for (int e = threadIdx.x; e < g.tile_elems; e += blockDim.x) {
            int64_t off = 0;
            int rem = e;
#pragma unroll
            for (int d = D - 1; d >= 0; --d) {
                const int i = rem % g.P[d];
                rem /= g.P[d];
                const AxisDev& a = t.ax[d];
                int64_t gi = org[d] + i;
                if (a.periodic) {
                    gi %= a.n;
                } else if (gi >= a.n) {
                    gi = a.n - 1;
                }
                off += gi * a.stride;
            }
            tile[e] = __ldg(cp + off);
        }
        __syncthreads();
        for (int64_t rr = r + threadIdx.x; rr < end; rr += blockDim.x) {
            const uint32_t idx = __ldg(ridx + rr);
            const uint32_t packed = __ldg(rcell + rr);
            int64_t c[D];
            int toff[D];
            float u[D];
            float base[D][W];
            int t0 = 0;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const int cl = static_cast<int>((packed >> g.shift[d]) & ((1u << g.lb[d]) - 1u));
                c[d] = org[d] + cl + O;
                u[d] = __ldg(ru + d * cap + rr);
                toff[d] = cl * g.tstride[d];
                t0 += toff[d];
                axis_weights32<O>(t.ax[d], c[d], u[d], 0, base[d]);
            }
            // centred contraction: weights of a value sum to 1, of a
            // derivative to 0, so FP32 weight rounding only scales the local
            // variation of the control points
            int tc = 0;
#pragma unroll
            for (int d = 0; d < D; ++d) tc += toff[d] + (W / 2) * g.tstride[d];
            const float c_ref = tile[tc];
            for (int k = 0; k < K; ++k) {
                float w[D][W];
                bool zero = false, value_out = true;
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    const int kd = plan.ord[k][d];
                    if (kd != 0) value_out = false;
                    if (kd > O) {
                        zero = true;
                    } else if (kd == 0) {
#pragma unroll
                        for (int i = 0; i < W; ++i) w[d][i] = base[d][i];
                    } else {
                        axis_weights32<O>(t.ax[d], c[d], u[d], kd, w[d]);
                    }
                }
                float acc = 0.0f;
                if (!zero) {
#pragma unroll
                    for (int rw = 0; rw < ROWS; ++rw) {
                        int o = t0;
                        float wr = 1.0f;
                        int rem = rw;
#pragma unroll
                        for (int d = D - 2; d >= 0; --d) {
                            const int i = rem % W;
                            rem /= W;
                            o += i * g.tstride[d];
                            wr *= w[d][i];
                        }
                        float s = 0.0f;
#pragma unroll
                        for (int i = 0; i < W; ++i) s += w[D - 1][i] * (tile[o + i] - c_ref);
                        acc += wr * s;
                    }
                    if (value_out) acc += c_ref;
                }
                if (out_f32)
                    static_cast<float*>(out)[static_cast<int64_t>(idx) * K + k] = acc;
                else
                    static_cast<double*>(out)[static_cast<int64_t>(idx) * K + k] = static_cast<double>(acc);
            }
        }
        r = end;
    }
}

}  // namespace bin_detail
}  // namespace intp_gb300
