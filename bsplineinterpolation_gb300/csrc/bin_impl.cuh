// Binned evaluation (mixed form): queries are counting-sorted by spatial
// bucket, then every bucket is evaluated against a shared-memory tile of the
// control points it touches.
//
// Random queries gathered straight from a 256^3 table touch ~22 sectors each
// and run at L1/L2 gather speed; after binning, the (O+1)^D neighbourhood of
// every query of a bucket comes from one tile of prod(B_d + O) control points
// staged once in shared memory.
//
//   locate:  exact span (integer keys) and FP32 local offsets of every query,
//            one 8- or 16-byte record per query in input order, and
//            per-(bucket, CTA) counts
//   scan:    exclusive prefix sum over (bucket, CTA) -> first slot of each pair
//   permute: every record moves to its pair's next slot (one vector store)
//   eval:    CTA j takes the j-th equal slice of the sorted records, stages the
//            tile of each bucket it meets with asynchronous copies, evaluates,
//            writes out[index]
//
// Locate and permute aggregate their shared-memory atomics per warp
// (__match_any_sync): lanes of a warp that fall into one bucket take
// consecutive slots with a single atomic, so clustered queries neither
// serialise on a counter nor scatter their records.
//
// Queries are processed in chunks of the input. A chunk is large (millions of
// queries) so each bucket's tile is staged a few times per chunk only; its
// output writes land in a region small enough to stay in L2 until its
// sectors are complete.
#pragma once

#include <cuda.h>

#include <cstdint>

#include "async_copy.cuh"
#include "basis32.cuh"
#include "device_common.cuh"
#include "launch.hpp"
#include "mixed_point.cuh"

namespace intp_gb300 {
namespace bin_detail {

constexpr int kBinThreads = 256;   // evaluation CTA
constexpr int kSortThreads = 512;  // count / scatter CTA

// Exact span and FP32 local offset of one coordinate on axis a (mixed form),
// with 32-bit span indices (binned tables have fewer than 2^31 knots per
// axis).
__device__ __forceinline__ int span_and_offset(const AxisDev& a, int order, double x, float& u) {
    if (a.periodic) x = periodic_wrap(a, x);
    float xh, xl;
    split_double(x, xh, xl);
    const int h = a.uniform ? uniform_hint32(a, xh) : order;
    const int c = locate_span32(a, order, knot_key(x), h);
    u = (xh - __ldg(a.khi + c)) + (xl - __ldg(a.klo + c));
    return c;
}

template <int D>
__device__ __forceinline__ uint32_t bucket_of(const BinGeom& g, const int (&cl)[D]) {
    uint32_t b = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) b = b * static_cast<uint32_t>(g.nb[d]) + static_cast<uint32_t>(cl[d] >> g.lb[d]);
    return b;
}

// Query records: u_0 .. u_{D-1} (FP32 local offsets) in the first words and a
// tag word last, 8 bytes for D = 1 and 16 bytes otherwise, so each record
// moves with one vector access. The tag holds the query's local span within
// its bucket in its low kCellBits bits (B_d = 2^lb[d] spans per axis,
// sum lb[d] = 12 for every D) and, above them, the bucket (records in input
// order) or the query's index within its sort CTA's input slice (records in
// bucket order).
constexpr int kCellBits = 12;
constexpr int kMaxSortBlocks = 1024;
constexpr int64_t kMaxSlice = int64_t{1} << (32 - kCellBits);

template <int D>
__host__ __device__ constexpr int rec_words() {
    return D == 1 ? 2 : 4;
}

template <int D>
struct RecVec {
    using type = uint4;
};
template <>
struct RecVec<1> {
    using type = uint2;
};

template <int D>
__device__ __forceinline__ void rec_store(uint32_t* rec, int64_t slot, const float (&u)[D], uint32_t tag) {
    if constexpr (D == 1) {
        reinterpret_cast<uint2*>(rec)[slot] = make_uint2(__float_as_uint(u[0]), tag);
    } else {
        uint4 v;
        v.x = __float_as_uint(u[0]);
        v.y = __float_as_uint(u[1]);
        v.z = 0u;
        if constexpr (D >= 3) v.z = __float_as_uint(u[2]);
        v.w = tag;
        reinterpret_cast<uint4*>(rec)[slot] = v;
    }
}

template <int D>
__device__ __forceinline__ void rec_load(const uint32_t* rec, int64_t slot, uint32_t (&w)[rec_words<D>()]) {
    if constexpr (D == 1) {
        const uint2 v = __ldg(reinterpret_cast<const uint2*>(rec) + slot);
        w[0] = v.x;
        w[1] = v.y;
    } else {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(rec) + slot);
        w[0] = v.x;
        w[1] = v.y;
        w[2] = v.z;
        w[3] = v.w;
    }
}

// Counting sort without global atomics. CTA `blk` owns the input slice
// [blk*S, (blk+1)*S) (S < 2^20).
//   locate:  exact spans and FP32 offsets of every query of the slice, one
//            record per query written in input order, and the slice's
//            per-bucket counts in blkcount[b * nblk + blk] (bucket-major);
//   scan:    exclusive prefix sum over (bucket, CTA): the first slot of every
//            pair (the first slot of bucket b is scan[b * nblk]);
//   permute: moves every record of the slice to its pair's next slot
//            (shared-memory cursors).
// Shared-memory atomics are aggregated per warp (__match_any_sync), and every
// thread runs the same number of loop trips so the match sees all lanes.
template <int D>
__global__ void __launch_bounds__(kSortThreads) locate_kernel(TableDev t, BinGeom g, const double* __restrict__ coords,
                                                             int64_t n, int64_t slice, uint32_t* __restrict__ in_rec,
                                                             uint32_t* __restrict__ blkcount) {
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
            int cl[D];
            float u[D];
            uint32_t cell = 0;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                cl[d] = span_and_offset(t.ax[d], t.order, __ldg(coords + p * D + d), u[d]) - t.order;
                cell |= static_cast<uint32_t>(cl[d] & ((1 << g.lb[d]) - 1)) << g.shift[d];
            }
            b = bucket_of<D>(g, cl);
            rec_store<D>(in_rec, p, u, (b << kCellBits) | cell);
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, b);
        if (valid && lane == __ffs(peers) - 1) atomicAdd(&sh_count[b], static_cast<uint32_t>(__popc(peers)));
    }
    __syncthreads();
    for (int64_t b = threadIdx.x; b < g.nbuckets; b += blockDim.x) blkcount[b * nblk + blk] = sh_count[b];
}

template <int D>
__global__ void __launch_bounds__(kSortThreads) permute_kernel(BinGeom g, int64_t n, int64_t slice,
                                                              const uint32_t* __restrict__ in_rec,
                                                              const uint32_t* __restrict__ blkoffset,
                                                              uint32_t* __restrict__ rec) {
    extern __shared__ uint32_t sh_cursor[];
    constexpr int RW = rec_words<D>();
    const int nblk = gridDim.x, blk = blockIdx.x;
    for (int64_t b = threadIdx.x; b < g.nbuckets; b += blockDim.x) sh_cursor[b] = blkoffset[b * nblk + blk];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const int64_t p0 = blk * slice, p1 = (p0 + slice < n) ? p0 + slice : n;
    constexpr uint32_t cell_mask = (1u << kCellBits) - 1u;
    for (int64_t base = p0; base < p1; base += blockDim.x) {
        const int64_t p = base + threadIdx.x;
        const bool valid = p < p1;
        uint32_t w[RW];
        uint32_t b = 0xFFFFFFFFu;
        if (valid) {
            rec_load<D>(in_rec, p, w);
            b = w[RW - 1] >> kCellBits;
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, b);
        const int leader = __ffs(peers) - 1;
        uint32_t first = 0;
        if (valid && lane == leader) first = atomicAdd(&sh_cursor[b], static_cast<uint32_t>(__popc(peers)));
        first = __shfl_sync(0xFFFFFFFFu, first, leader);
        if (valid) {
            const uint32_t slot = first + static_cast<uint32_t>(__popc(peers & lt_mask));
            w[RW - 1] = (static_cast<uint32_t>(p - p0) << kCellBits) | (w[RW - 1] & cell_mask);
            if constexpr (D == 1)
                reinterpret_cast<uint2*>(rec)[slot] = make_uint2(w[0], w[1]);
            else
                reinterpret_cast<uint4*>(rec)[slot] = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
}

constexpr int ipow_c(int b, int e) { return e == 0 ? 1 : b * ipow_c(b, e - 1); }

// Compile-time tile shape: P_d = 2^bucket_log2 + O positions per axis,
// row-major, rows of the last axis padded to a multiple of 4 floats (the
// 16-byte inner extent of a TMA box).
template <int D, int O>
struct TileShape {
    static constexpr int P(int d) { return (1 << bucket_log2(D, d)) + O; }
    static constexpr int PL() { return (P(D - 1) + 3) & ~3; }
    static constexpr int S(int d) { return d >= D - 1 ? 1 : (d == D - 2 ? PL() : P(d + 1) * S(d + 1)); }
    static constexpr int elems() { return D == 1 ? PL() : P(0) * S(0); }
};

// Offset (floats) of the remainders' tile after the control points' tile,
// keeping it 128-byte aligned; the launchers size the dynamic shared memory
// the same way.
template <class TS>
constexpr int tile_lo_offset() {
    return (TS::elems() + 31) & ~31;
}

// Control-point index along axis a of tile position org + i (periodic wrap,
// clamp at the end of a non-periodic axis: positions past the last control
// point are never read by a query of the bucket).
__device__ __forceinline__ int tile_index(const AxisDev& a, int gi) {
    const int n = static_cast<int>(a.n);
    return a.periodic ? gi % n : (gi < n ? gi : n - 1);
}

// Outputs of one query for a plan whose outputs differ only in their axis-0
// derivative order (DerivPlan::simple): the contraction over axes 1..D-1 is
// done once, then each output applies its own axis-0 weights. Weights come
// from axis_weights32 (compile-time polynomials on uniform interior spans,
// knot tables elsewhere). The arithmetic is that of mixed_point_outputs on
// the same inputs (same weight code, same summation order), so results are
// identical.
template <int D, int O, class TS, class Emit>
__device__ __forceinline__ void lean_point(const TableDev& t, const int (&c)[D], const float (&u)[D], const float* tl,
                                           const DerivPlan& plan, float cref, float cbase, const Emit& emit) {
    constexpr int W = O + 1;
    constexpr int ROWS1 = D >= 2 ? ipow_c(W, D - 2) : 1;
    float w[D][W];
#pragma unroll
    for (int d = 1; d < D; ++d) axis_weights32<O>(t.ax[d], c[d], u[d], 0, w[d]);
    float Pz[W];
#pragma unroll
    for (int i0 = 0; i0 < W; ++i0) {
        float acc = 0.0f;
#pragma unroll
        for (int rw = 0; rw < ROWS1; ++rw) {
            int off = i0 * TS::S(0);
            float wr = 1.0f;
            int rem = rw;
#pragma unroll
            for (int d = D - 2; d >= 1; --d) {
                const int i = rem % W;
                rem /= W;
                wr *= w[d][i];
                off += i * TS::S(d);
            }
            if constexpr (D == 1) {
                acc = tl[off] - cref;
            } else {
                float s = 0.0f;
#pragma unroll
                for (int i = 0; i < W; ++i) s += w[D - 1][i] * (tl[off + i] - cref);
                acc += wr * s;
            }
        }
        Pz[i0] = acc;
    }
    const int K = plan.k;
    for (int k = 0; k < K; ++k) {
        const int k0 = plan.ord[k][0];
        float v = 0.0f;
        if (k0 <= O) {
            float wl[W];
            axis_weights32<O>(t.ax[0], c[0], u[0], k0, wl);
#pragma unroll
            for (int i = 0; i < W; ++i) v += wl[i] * Pz[i];
            if (k0 == 0) v = (v + cref) + cbase;
        }
        emit(k, v);
    }
}

// Evaluation of the records of one bucket [r, end) against its staged tile.
// seg[j] is the first slot of the bucket's records from sort CTA j (nblk
// entries); a record's query index is j * slice + its local index.
// LEAN: a DerivPlan::simple plan.
template <int D, int O, bool LEAN, class TS>
__device__ __forceinline__ void eval_records(const TableDev& t, const BinGeom& g, const DerivPlan& plan,
                                             const float* tile, const int (&org)[D], float cbase,
                                             const uint32_t* seg, int nblk, int64_t slice,
                                             const uint32_t* __restrict__ rec, int64_t r, int64_t end,
                                             void* __restrict__ out, int out_f32) {
    constexpr int RW = rec_words<D>();
    constexpr int W = O + 1;
    const int K = plan.k;
    // records are software-pipelined: the next one loads while the current
    // one is evaluated
    uint32_t nx[RW];
    int64_t rr = r + threadIdx.x;
    if (rr < end) rec_load<D>(rec, rr, nx);
    for (; rr < end; rr += blockDim.x) {
        uint32_t cur[RW];
#pragma unroll
        for (int j = 0; j < RW; ++j) cur[j] = nx[j];
        const int64_t nr = rr + blockDim.x;
        if (nr < end) rec_load<D>(rec, nr, nx);
        const uint32_t tag = cur[RW - 1];
        // sort CTA of the record: the last segment starting at or before rr
        int lo = 0, hi = nblk;
        const uint32_t slot = static_cast<uint32_t>(rr);
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (seg[mid] <= slot)
                lo = mid;
            else
                hi = mid;
        }
        const int64_t idx = static_cast<int64_t>(lo) * slice + (tag >> kCellBits);
        int tb = 0;
        int cl[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            cl[d] = static_cast<int>((tag >> g.shift[d]) & ((1u << bucket_log2(D, d)) - 1u));
            tb += cl[d] * TS::S(d);
        }
        const float* tl = tile + tb;
        // the query's reference: its central control point
        int tref = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) tref += ref_tap<O>() * TS::S(d);
        const float cref = tl[tref];
        const int64_t o0 = idx * K;
        auto emit = [out, out_f32, o0](int k, float v) {
            if (out_f32)
                static_cast<float*>(out)[o0 + k] = v;
            else
                static_cast<double*>(out)[o0 + k] = static_cast<double>(v);
        };
        if constexpr (LEAN) {
            float u[D];
            int c[D];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                u[d] = __uint_as_float(cur[d]);
                c[d] = org[d] + cl[d] + O;
            }
            lean_point<D, O, TS>(t, c, u, tl, plan, cref, cbase, emit);
        } else {
            float u[D];
            int64_t c[D];
            float base[D][W];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                u[d] = __uint_as_float(cur[d]);
                c[d] = org[d] + cl[d] + O;
                axis_weights32<O>(t.ax[d], c[d], u[d], 0, base[d]);
            }
            mixed_point_outputs<D, O>(
                t, plan, c, u, base, cref, cbase,
                [tl, cref](const int (&ix)[D]) {
                    int off = 0;
#pragma unroll
                    for (int d = 0; d < D; ++d) off += ix[d] * TS::S(d);
                    return tl[off] - cref;
                },
                emit);
        }
    }
}

// The general path, out of line: its register pressure (runtime derivative
// plans, table-driven weights at clamped or non-uniform spans) stays out of
// the lean path's allocation.
template <int D, int O, class TS>
__device__ __noinline__ void eval_records_general(const TableDev& t, const BinGeom& g, const DerivPlan& plan,
                                                  const float* tile, const int (&org)[D], float cbase,
                                                  const uint32_t* seg, int nblk, int64_t slice,
                                                  const uint32_t* __restrict__ rec, int64_t r, int64_t end,
                                                  void* __restrict__ out, int out_f32) {
    eval_records<D, O, false, TS>(t, g, plan, tile, org, cbase, seg, nblk, slice, rec, r, end, out, out_f32);
}

template <int D, int O>
__global__ void __launch_bounds__(kBinThreads, 2) eval_kernel(TableDev t, BinGeom g, const uint32_t* __restrict__ blkoffset,
                                                           int nblk, int64_t slice, const uint32_t* __restrict__ rec,
                                                           int64_t nrec, DerivPlan plan, void* __restrict__ out,
                                                           int out_f32, const __grid_constant__ CUtensorMap tmap,
                                                           const __grid_constant__ CUtensorMap tmap_lo,
                                                           int use_tma) {
    using TS = TileShape<D, O>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // 128-byte aligned tiles (TMA destinations): the control points, then
    // their remainders when the table keeps them
    float* tile = reinterpret_cast<float*>(smem_raw + ((128 - (smem_addr(smem_raw) & 127)) & 127));
    float* tile_lo = tile + tile_lo_offset<TS>();
    // remainders staged for derivative requests only (as in the direct kernel)
    const float* __restrict__ cl = plan.has_deriv ? t.ctrl_lo : nullptr;
    __shared__ __align__(8) uint64_t sh_bar;
    __shared__ float sh_cbase;
    __shared__ DerivPlan sh_plan;  // indexed by runtime output / group numbers
    __shared__ TableDev sh_t;      // passed by reference to the out-of-line path
    __shared__ int sh_last[TS::P(D - 1)];                          // last-axis control-point indices
    __shared__ int64_t sh_outer[D > 1 ? D - 1 : 1][D > 1 ? TS::P(0) : 1];  // outer-axis offsets
    __shared__ uint32_t sh_seg[kMaxSortBlocks];                    // the bucket's per-CTA first slots
    const float* __restrict__ cp = static_cast<const float*>(t.ctrl);
    const int64_t r0 = nrec * blockIdx.x / gridDim.x, r1 = nrec * (blockIdx.x + 1) / gridDim.x;
    if (r0 >= r1) return;
    if (threadIdx.x == 0) {
        sh_plan = plan;
        sh_t = t;
        mbar_init(&sh_bar, 1);
    }
    __syncthreads();
    uint32_t bar_phase = 0;
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
    constexpr int PL = TS::P(D - 1);  // tile row length (last axis)
    constexpr int PLP = TS::PL();      // its padded pitch
    while (r < r1) {
        while (bstart(b + 1) <= r) ++b;
        const int64_t bend = bstart(b + 1);
        const int64_t end = bend < r1 ? bend : r1;
        int org[D];
        {
            int rem = static_cast<int>(b);
#pragma unroll
            for (int d = D - 1; d >= 0; --d) {
                org[d] = (rem % g.nb[d]) << bucket_log2(D, d);
                rem /= g.nb[d];
            }
        }
        __syncthreads();
        for (int j = threadIdx.x; j < nblk; j += kBinThreads) sh_seg[j] = __ldg(blkoffset + b * nblk + j);
        if (threadIdx.x == 0 && cl) {
            // the operands' base: the control point at the tile's centre
            // (clamped at the end of a non-periodic axis, as in the direct
            // kernel)
            int64_t off = 0;
#pragma unroll
            for (int d = 0; d < D; ++d)
                off += static_cast<int64_t>(tile_index(t.ax[d], org[d] + TS::P(d) / 2)) * t.ax[d].stride;
            sh_cbase = __ldg(cp + off);
        }
        // one TMA box unless the tile wraps around a periodic axis
        bool tma = use_tma != 0;
#pragma unroll
        for (int d = 0; d < D; ++d)
            if (t.ax[d].periodic && org[d] + TS::P(d) > t.ax[d].n) tma = false;
        if (tma) {
            if (threadIdx.x == 0) {
                fence_async_smem();  // the tiles' earlier generic-proxy accesses before the async write
                mbar_expect_tx(&sh_bar, static_cast<uint32_t>(TS::elems() * 4 * (cl ? 2 : 1)));
                if constexpr (D == 3) tma_load_3d(tile, &tmap, org[2], org[1], org[0], &sh_bar);
                if constexpr (D == 2) tma_load_2d(tile, &tmap, org[1], org[0], &sh_bar);
                if (cl) {
                    if constexpr (D == 3) tma_load_3d(tile_lo, &tmap_lo, org[2], org[1], org[0], &sh_bar);
                    if constexpr (D == 2) tma_load_2d(tile_lo, &tmap_lo, org[1], org[0], &sh_bar);
                }
            }
            const bool ok = mbar_wait(&sh_bar, bar_phase);
            if (!__syncthreads_and(ok)) {
                if (!ok) mbar_wait(&sh_bar, bar_phase);  // bounded: let the copy in flight land
                return;
            }
            bar_phase ^= 1u;
        } else {
            // per-axis global offsets of the tile positions (periodic wrap,
            // clamp at the end of a non-periodic axis)
            for (int i = threadIdx.x; i < PL; i += kBinThreads) sh_last[i] = tile_index(t.ax[D - 1], org[D - 1] + i);
            if constexpr (D >= 2) {
                for (int i = threadIdx.x; i < TS::P(0); i += kBinThreads)
                    sh_outer[0][i] = static_cast<int64_t>(tile_index(t.ax[0], org[0] + i)) * t.ax[0].stride;
            }
            if constexpr (D >= 3) {
                for (int i = threadIdx.x; i < TS::P(1); i += kBinThreads)
                    sh_outer[1][i] = static_cast<int64_t>(tile_index(t.ax[1], org[1] + i)) * t.ax[1].stride;
            }
            __syncthreads();
            // asynchronous element copies, all in flight at once
            for (int e = threadIdx.x; e < TS::elems(); e += kBinThreads) {
                int rem = e;
                const int il = rem % PLP;
                rem /= PLP;
                if (il >= PL) continue;  // row padding
                int64_t off = sh_last[il];
#pragma unroll
                for (int d = D - 2; d >= 0; --d) {
                    const int i = rem % TS::P(d);
                    rem /= TS::P(d);
                    off += sh_outer[d][i];
                }
                cp_async<4>(tile + e, cp + off);
                if (cl) cp_async<4>(tile_lo + e, cl + off);
            }
            cp_async_wait_all();
        }
        __syncthreads();
        // operands, once per tile element: the stored FP32 control point, or
        // with remainders (ctrl - cbase) + ctrl_lo; each query then reads them
        // relative to its own central tap
        float cbase = 0.0f;
        if (cl) {
            cbase = sh_cbase;
            for (int e = threadIdx.x; e < TS::elems(); e += kBinThreads) tile[e] = (tile[e] - cbase) + tile_lo[e];
            __syncthreads();
        }
        if (sh_plan.simple)
            eval_records<D, O, true, TS>(sh_t, g, sh_plan, tile, org, cbase, sh_seg, nblk, slice, rec, r, end, out,
                                         out_f32);
        else
            eval_records_general<D, O, TS>(sh_t, g, sh_plan, tile, org, cbase, sh_seg, nblk, slice, rec, r, end, out,
                                           out_f32);
        r = end;
    }
}

}  // namespace bin_detail
}  // namespace intp_gb300
