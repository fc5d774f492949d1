// Binned evaluation (mixed form): queries are counting-sorted by spatial
// bucket, then every bucket is evaluated against a shared-memory tile of the
// control points it touches.
//
// Random queries gathered straight from a 256^3 table touch ~22 sectors each
// and run at L1/L2 gather speed; after binning, the (O+1)^D neighbourhood of
// every query of a bucket comes from one tile of prod(B_d + O) control points
// staged once in shared memory.
//
//   count:   exact spans of every query of a sort CTA's input slice, and the
//            slice's per-bucket counts (per-(bucket, CTA) pairs)
//   scan:    exclusive prefix sum over (bucket, CTA) -> first slot of each pair
//   scatter: the same CTA recomputes each query's record (spans and FP32
//            local offsets) and writes it to the next free slot of its pair
//   eval:    CTA j takes the j-th equal slice of the sorted records, stages the
//            tile of each bucket it meets with asynchronous copies, evaluates,
//            writes out[index]
//
// Count and scatter aggregate their shared-memory atomics per warp
// (__match_any_sync): lanes of a warp that fall into one bucket take
// consecutive slots with a single atomic, so clustered queries neither
// serialise on a counter nor scatter their records. Recomputing the records
// costs less than writing them in input order and moving them: a record is
// written once (16 bytes per query) and read once.
//
// Queries are processed in chunks of the input, as large as a record's
// 20-bit slice index allows (up to 2^28 queries): each bucket's tile is staged
// once per evaluation CTA that meets the bucket, so the more queries one sort
// holds, the more of them share each staged tile.
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
constexpr int kLocateThreads = 768;  // count CTA (two per SM at up to 42 registers)
constexpr int kSortThreads = 768;    // scatter CTA (two per SM at up to 42 registers)

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
constexpr int kMaxSortBlocks = 512;
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

// Records of every query of the slice in input order, and the slice's
// per-(bucket, CTA) counts: the read-out of the binned path's spans
// (intp_locate_binned) decodes these records. Same spans and offsets as the
// count and scatter kernels (span_and_offset).
template <int D>
__global__ void __launch_bounds__(kLocateThreads, 2) locate_kernel(TableDev t, BinGeom g, const double* __restrict__ coords,
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
        // one atomic per group of lanes with the same bucket
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, b);
        const int leader = __ffs(peers) - 1;
        if (valid && lane == leader) atomicAdd(&sh_count[b], static_cast<uint32_t>(__popc(peers)));
    }
    __syncthreads();
    for (int64_t b = threadIdx.x; b < g.nbuckets; b += blockDim.x) blkcount[b * nblk + blk] = sh_count[b];
}

// Counting pass of the two-pass sort (count_kernel, then scatter_kernel): the
// per-(bucket, CTA) counts of the slice, from the same exact spans as
// locate_kernel, writing no records.
template <int D>
__global__ void __launch_bounds__(kLocateThreads, 2) count_kernel(TableDev t, BinGeom g, const double* __restrict__ coords,
                                                            int64_t n, int64_t slice,
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
#pragma unroll
            for (int d = 0; d < D; ++d) {
                float u;
                cl[d] = span_and_offset(t.ax[d], t.order, __ldg(coords + p * D + d), u) - t.order;
            }
            b = bucket_of<D>(g, cl);
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, b);
        const int leader = __ffs(peers) - 1;
        if (valid && lane == leader) atomicAdd(&sh_count[b], static_cast<uint32_t>(__popc(peers)));
    }
    __syncthreads();
    for (int64_t b = threadIdx.x; b < g.nbuckets; b += blockDim.x) blkcount[b * nblk + blk] = sh_count[b];
}

// Scatter pass of the two-pass sort: CTA blk recomputes the record of every
// query of its slice (the same spans and offsets as the counting pass) and
// writes it to the next free slot of its (bucket, CTA) pair, taken from a
// shared-memory cursor that starts at the pair's first slot (warp-aggregated
// atomics). The order of records within a pair depends on timing; each
// query's outputs do not. The tag holds the query's index within the slice
// (the evaluation finds the slice from the pair the slot lies in).
template <int D>
__global__ void __launch_bounds__(kSortThreads, 2) scatter_kernel(TableDev t, BinGeom g, const double* __restrict__ coords,
                                                              int64_t n, int64_t slice,
                                                              const uint32_t* __restrict__ blkoffset,
                                                              uint32_t* __restrict__ rec) {
    extern __shared__ uint32_t sh_cursor[];
    const int nblk = gridDim.x, blk = blockIdx.x;
    for (int64_t b = threadIdx.x; b < g.nbuckets; b += blockDim.x) sh_cursor[b] = __ldg(blkoffset + b * nblk + blk);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t p0 = blk * slice, p1 = (p0 + slice < n) ? p0 + slice : n;
    for (int64_t base = p0; base < p1; base += blockDim.x) {
        const int64_t p = base + threadIdx.x;
        const bool valid = p < p1;
        uint32_t b = 0xFFFFFFFFu, cell = 0;
        float u[D];
        if (valid) {
            int cl[D];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                cl[d] = span_and_offset(t.ax[d], t.order, __ldg(coords + p * D + d), u[d]) - t.order;
                cell |= static_cast<uint32_t>(cl[d] & ((1 << g.lb[d]) - 1)) << g.shift[d];
            }
            b = bucket_of<D>(g, cl);
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, b);
        const int leader = __ffs(peers) - 1;
        uint32_t first = 0;
        if (valid && lane == leader) first = atomicAdd(&sh_cursor[b], static_cast<uint32_t>(__popc(peers)));
        first = __shfl_sync(0xFFFFFFFFu, first, leader);
        if (valid) {
            const uint32_t slot = first + static_cast<uint32_t>(__popc(peers & ((1u << lane) - 1u)));
            rec_store<D>(rec, slot, u, (static_cast<uint32_t>(p - p0) << kCellBits) | cell);
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

// Shared-memory plan of the evaluation CTA for one (D, O): the control
// points' tile; a second region of the same size that holds the remainders'
// tile while a bucket is staged and then a piece of the bucket's records
// sorted by cell; the cell of every sorted record; and the per-cell counters
// of the piece (two 16-bit counts per word).
template <int D, int O>
struct EvalSmem {
    using TS = TileShape<D, O>;
    static constexpr int kRecBytes = rec_words<D>() * 4;
    static constexpr int kTileBytes = (TS::elems() * 4 + 127) & ~127;
    static constexpr int kPiece = (kTileBytes / kRecBytes) / kBinThreads * kBinThreads;
    static constexpr int kPerThread = kPiece / kBinThreads;
    static constexpr int kCellofBytes = (kPiece * 2 + 127) & ~127;
    static constexpr int kCountWords = (1 << kCellBits) / 2;
    static constexpr int kBytes = 2 * kTileBytes + kCellofBytes + kCountWords * 4 + 128;
    static_assert(kPiece >= kBinThreads && kPiece < 65536, "piece of the in-CTA sort");
};

// Exclusive scan, in place, of the 2^kCellBits 16-bit cell counts packed two
// per word (cell 2w in the low half of word w): afterwards each half holds
// the first sorted position of its cell's records in the piece (< 2^16).
__device__ __forceinline__ void scan_cell_counts(uint32_t* cnt, uint32_t* warp_sums) {
    constexpr int kWords = (1 << kCellBits) / 2;
    constexpr int kPer = kWords / kBinThreads;  // words per thread
    static_assert(kPer * kBinThreads == kWords && kPer % 4 == 0, "cell counter layout");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t v[kPer];
#pragma unroll
    for (int j = 0; j < kPer; j += 4) {
        const uint4 q = reinterpret_cast<const uint4*>(cnt + tid * kPer)[j / 4];
        v[j] = q.x;
        v[j + 1] = q.y;
        v[j + 2] = q.z;
        v[j + 3] = q.w;
    }
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < kPer; ++j) sum += (v[j] & 0xFFFFu) + (v[j] >> 16);
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    uint32_t run = incl - sum;
    for (int w = 0; w < warp; ++w) run += warp_sums[w];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        const uint32_t lo = v[j] & 0xFFFFu, hi = v[j] >> 16;
        v[j] = run | ((run + lo) << 16);
        run += lo + hi;
    }
#pragma unroll
    for (int j = 0; j < kPer; j += 4)
        reinterpret_cast<uint4*>(cnt + tid * kPer)[j / 4] = make_uint4(v[j], v[j + 1], v[j + 2], v[j + 3]);
}

// Outputs of one sorted record: w = (u_0 .. u_{D-1} as FP32, query index),
// cell = its span within the bucket (packed as in the tag).
template <int D, int O, bool LEAN, class TS>
__device__ __forceinline__ void eval_record(const TableDev& t, const BinGeom& g, const DerivPlan& plan,
                                            const float* tile, const int (&org)[D], float cbase,
                                            const uint32_t (&w)[rec_words<D>()], uint32_t cell,
                                            void* __restrict__ out, int out_f32, int C, int ch) {
    constexpr int RW = rec_words<D>();
    constexpr int W = O + 1;
    const int K = plan.k;
    const int64_t idx = static_cast<int64_t>(w[RW - 1]);
    int tb = 0;
    int cl[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
        cl[d] = static_cast<int>((cell >> g.shift[d]) & ((1u << bucket_log2(D, d)) - 1u));
        tb += cl[d] * TS::S(d);
    }
    const float* tl = tile + tb;
    // the query's reference: its central control point
    int tref = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) tref += ref_tap<O>() * TS::S(d);
    const float cref = tl[tref];
    const int64_t o0 = idx * K;
    // value and one derivative (the common request) leave as one 8-byte store;
    // output k of channel ch of a vector-valued table goes to (o0 + k) * C + ch
    float first = 0.0f;
    const bool pair = out_f32 == 3 && K == 2 && C == 1;
    auto emit = [out, out_f32, o0, pair, C, ch, &first](int k, float v) {
        if (pair) {
            if (k == 0)
                first = v;
            else
                reinterpret_cast<float2*>(static_cast<float*>(out) + o0)[0] = make_float2(first, v);
        } else if (out_f32) {
            static_cast<float*>(out)[(o0 + k) * C + ch] = v;
        } else {
            static_cast<double*>(out)[(o0 + k) * C + ch] = static_cast<double>(v);
        }
    };
    if constexpr (LEAN) {
        float u[D];
        int c[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            u[d] = __uint_as_float(w[d]);
            c[d] = org[d] + cl[d] + O;
        }
        lean_point<D, O, TS>(t, c, u, tl, plan, cref, cbase, emit);
    } else {
        float u[D];
        int64_t c[D];
        float base[D][W];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            u[d] = __uint_as_float(w[d]);
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

// Evaluation of the n records of a piece, in cell order (sorted positions
// tid, tid + kBinThreads, ...: the lanes of a warp read the same or
// neighbouring cells of the tile).
template <int D, int O, bool LEAN, class TS>
__device__ __forceinline__ void eval_sorted(const TableDev& t, const BinGeom& g, const DerivPlan& plan,
                                            const float* tile, const int (&org)[D], float cbase,
                                            const uint32_t* sbuf, const uint16_t* cellof, int n,
                                            void* __restrict__ out, int out_f32, int C, int ch) {
    constexpr int RW = rec_words<D>();
    for (int q = threadIdx.x; q < n; q += kBinThreads) {
        uint32_t w[RW];
        if constexpr (RW == 2) {
            const uint2 v = reinterpret_cast<const uint2*>(sbuf)[q];
            w[0] = v.x;
            w[1] = v.y;
        } else {
            const uint4 v = reinterpret_cast<const uint4*>(sbuf)[q];
            w[0] = v.x;
            w[1] = v.y;
            w[2] = v.z;
            w[3] = v.w;
        }
        eval_record<D, O, LEAN, TS>(t, g, plan, tile, org, cbase, w, cellof[q], out, out_f32, C, ch);
    }
}

// The general path, out of line: its register pressure (runtime derivative
// plans, table-driven weights at clamped or non-uniform spans) stays out of
// the lean path's allocation.
template <int D, int O, class TS>
__device__ __noinline__ void eval_sorted_general(const TableDev& t, const BinGeom& g, const DerivPlan& plan,
                                                 const float* tile, const int (&org)[D], float cbase,
                                                 const uint32_t* sbuf, const uint16_t* cellof, int n,
                                                 void* __restrict__ out, int out_f32, int C, int ch) {
    eval_sorted<D, O, false, TS>(t, g, plan, tile, org, cbase, sbuf, cellof, n, out, out_f32, C, ch);
}

// Evaluation CTA. CTA j takes the j-th equal slice of the records in bucket
// order. For each bucket it meets it stages the bucket's tile (one TMA box,
// or element copies where the tile wraps around a periodic axis), then takes
// the bucket's records in pieces of kPiece: each piece is counting-sorted by
// cell in shared memory (16-bit counters, warp-aggregated atomics) and then
// evaluated in cell order. The cell packs row-major (last axis lowest), so
// lanes with neighbouring sorted records read neighbouring tile words.
template <int D, int O>
__global__ void __launch_bounds__(kBinThreads, 3) eval_kernel(TableDev t, BinGeom g, const uint32_t* __restrict__ blkoffset,
                                                           int nblk, int64_t slice, const uint32_t* __restrict__ rec,
                                                           int64_t nrec, DerivPlan plan, void* __restrict__ out,
                                                           int out_f32, const __grid_constant__ CUtensorMap tmap,
                                                           const __grid_constant__ CUtensorMap tmap_lo,
                                                           int use_tma) {
    using TS = TileShape<D, O>;
    using SM = EvalSmem<D, O>;
    constexpr int RW = rec_words<D>();
    constexpr int RPT = SM::kPerThread;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // 128-byte aligned regions: the tile (a TMA destination), the remainders'
    // tile / sorted records, the cells of the sorted records, the counters
    unsigned char* sm = smem_raw + ((128 - (smem_addr(smem_raw) & 127)) & 127);
    float* tile = reinterpret_cast<float*>(sm);
    float* tile_lo = reinterpret_cast<float*>(sm + SM::kTileBytes);
    uint32_t* sbuf = reinterpret_cast<uint32_t*>(sm + SM::kTileBytes);
    uint16_t* cellof = reinterpret_cast<uint16_t*>(sm + 2 * SM::kTileBytes);
    uint32_t* cnt = reinterpret_cast<uint32_t*>(sm + 2 * SM::kTileBytes + SM::kCellofBytes);
    // remainders staged for derivative requests only (as in the direct kernel)
    const float* __restrict__ cl = plan.has_deriv ? t.ctrl_lo : nullptr;
    __shared__ __align__(8) uint64_t sh_bar;
    __shared__ float sh_cbase;
    __shared__ DerivPlan sh_plan;  // indexed by runtime output / group numbers
    __shared__ TableDev sh_t;      // passed by reference to the out-of-line path
    __shared__ int sh_last[TS::P(D - 1)];                          // last-axis control-point indices
    __shared__ int64_t sh_outer[D > 1 ? D - 1 : 1][D > 1 ? TS::P(0) : 1];  // outer-axis offsets
    __shared__ uint32_t sh_seg[kMaxSortBlocks];                    // the bucket's per-sort-CTA first slots
    __shared__ uint32_t sh_warp[kBinThreads / 32];
    const float* __restrict__ cp = static_cast<const float*>(t.ctrl);
    const int C = t.channels > 1 ? t.channels : 1;
    const int64_t r0 = nrec * blockIdx.x / gridDim.x, r1 = nrec * (blockIdx.x + 1) / gridDim.x;
    if (r0 >= r1) return;
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    if (tid == 0) {
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
        // vector-valued tables: the bucket's records once per channel, each
        // channel's tile staged by element copies (the TMA maps cover one
        // channel)
        for (int ch = 0; ch < C; ++ch) {
        const float* __restrict__ cpc = cp + ch * t.chan_stride;
        const float* __restrict__ clc = cl ? cl + ch * t.chan_stride : nullptr;
        __syncthreads();
        for (int j = tid; j < nblk; j += kBinThreads) sh_seg[j] = __ldg(blkoffset + b * nblk + j);
        if (tid == 0 && cl) {
            // the operands' base: the control point at the tile's centre
            // (clamped at the end of a non-periodic axis, as in the direct
            // kernel)
            int64_t off = 0;
#pragma unroll
            for (int d = 0; d < D; ++d)
                off += static_cast<int64_t>(tile_index(t.ax[d], org[d] + TS::P(d) / 2)) * t.ax[d].stride;
            sh_cbase = __ldg(cpc + off);
        }
        // one TMA box unless the tile wraps around a periodic axis
        bool tma = use_tma != 0 && C == 1;
#pragma unroll
        for (int d = 0; d < D; ++d)
            if (t.ax[d].periodic && org[d] + TS::P(d) > t.ax[d].n) tma = false;
        if (tma) {
            if (tid == 0) {
                fence_async_smem();  // the tiles' earlier generic-proxy accesses before the async write
                mbar_expect_tx(&sh_bar, static_cast<uint32_t>(TS::elems() * 4 * (cl ? 2 : 1)));
                if constexpr (D == 3) tma_load_3d(tile, &tmap, org[2], org[1], org[0], &sh_bar);
                if constexpr (D == 2) tma_load_2d(tile, &tmap, org[1], org[0], &sh_bar);
                if (cl) {
                    if constexpr (D == 3) tma_load_3d(tile_lo, &tmap_lo, org[2], org[1], org[0], &sh_bar);
                    if constexpr (D == 2) tma_load_2d(tile_lo, &tmap_lo, org[1], org[0], &sh_bar);
                }
            }
            const uint32_t probes = g_tile_wait_probes;  // diagnostics: a forced short wait
            const bool ok = probes ? mbar_probe(&sh_bar, bar_phase, probes) : mbar_wait(&sh_bar, bar_phase);
            if (!__syncthreads_and(ok)) {
                if (!ok) mbar_wait(&sh_bar, bar_phase);  // bounded: let the copy in flight land
                return;
            }
            bar_phase ^= 1u;
        } else {
            // per-axis global offsets of the tile positions (periodic wrap,
            // clamp at the end of a non-periodic axis)
            for (int i = tid; i < PL; i += kBinThreads) sh_last[i] = tile_index(t.ax[D - 1], org[D - 1] + i);
            if constexpr (D >= 2) {
                for (int i = tid; i < TS::P(0); i += kBinThreads)
                    sh_outer[0][i] = static_cast<int64_t>(tile_index(t.ax[0], org[0] + i)) * t.ax[0].stride;
            }
            if constexpr (D >= 3) {
                for (int i = tid; i < TS::P(1); i += kBinThreads)
                    sh_outer[1][i] = static_cast<int64_t>(tile_index(t.ax[1], org[1] + i)) * t.ax[1].stride;
            }
            __syncthreads();
            // asynchronous element copies, all in flight at once
            for (int e = tid; e < TS::elems(); e += kBinThreads) {
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
                cp_async<4>(tile + e, cpc + off);
                if (cl) cp_async<4>(tile_lo + e, clc + off);
            }
            cp_async_wait_all();
        }
        __syncthreads();
        // operands, once per tile element: the stored FP32 control point, or
        // with remainders (ctrl - cbase) + ctrl_lo; each query then reads them
        // relative to its own central tap. The remainders' region is free
        // afterwards: it holds the sorted records of each piece.
        float cbase = 0.0f;
        if (cl) {
            cbase = sh_cbase;
            for (int e = tid; e < TS::elems(); e += kBinThreads) tile[e] = (tile[e] - cbase) + tile_lo[e];
        }
        int seg = 0;  // sort CTA of the thread's current record
        for (int64_t p0 = r; p0 < end; p0 += SM::kPiece) {
            const int n = static_cast<int>(end - p0 < SM::kPiece ? end - p0 : SM::kPiece);
            for (int wd = tid * 4; wd < SM::kCountWords; wd += kBinThreads * 4)
                *reinterpret_cast<uint4*>(cnt + wd) = make_uint4(0u, 0u, 0u, 0u);
            __syncthreads();
            // this thread's records: slots p0 + tid * RPT + i, in order. Their
            // tags first (all loads in flight); the whole records are read
            // again when they are placed (from L1: the tag's sector holds
            // the record)
            uint32_t key[RPT];   // cell | rank << 16
            uint32_t qidx[RPT];  // query index within the chunk
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                const int li = tid * RPT + i;
                qidx[i] = li < n ? __ldg(rec + (p0 + li) * RW + (RW - 1)) : 0u;
            }
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                const int li = tid * RPT + i;
                const bool valid = li < n;
                uint32_t cell = 0xFFFFFFFFu;
                if (valid) {
                    const uint32_t tag = qidx[i];
                    cell = tag & ((1u << kCellBits) - 1u);
                    // the record's sort CTA: the last segment starting at or
                    // before its slot (binary search once, then forward steps)
                    const uint32_t slot = static_cast<uint32_t>(p0 + li);
                    if (i == 0) {
                        int a = 0, z = nblk;
                        while (z - a > 1) {
                            const int mid = (a + z) >> 1;
                            if (sh_seg[mid] <= slot)
                                a = mid;
                            else
                                z = mid;
                        }
                        seg = a;
                    }
                    while (seg + 1 < nblk && sh_seg[seg + 1] <= slot) ++seg;
                    qidx[i] = static_cast<uint32_t>(static_cast<int64_t>(seg) * slice + (tag >> kCellBits));
                }
                // rank within the cell: one atomic per group of lanes with the
                // same cell
                const uint32_t peers = __match_any_sync(0xFFFFFFFFu, cell);
                const int leader = __ffs(peers) - 1;
                const uint32_t sh = (cell & 1u) * 16u;
                uint32_t old = 0;
                if (valid && lane == leader) old = atomicAdd(cnt + (cell >> 1), static_cast<uint32_t>(__popc(peers)) << sh);
                old = __shfl_sync(0xFFFFFFFFu, old, leader);
                const uint32_t rank = ((old >> sh) & 0xFFFFu) + static_cast<uint32_t>(__popc(peers & lt_mask));
                key[i] = (cell & 0xFFFFu) | (rank << 16);
            }
            __syncthreads();
            scan_cell_counts(cnt, sh_warp);
            __syncthreads();
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                const int li = tid * RPT + i;
                if (li < n) {
                    uint32_t w[RW];
                    rec_load<D>(rec, p0 + li, w);
                    w[RW - 1] = qidx[i];
                    const uint32_t cell = key[i] & 0xFFFFu;
                    const uint32_t q = ((cnt[cell >> 1] >> ((cell & 1u) * 16u)) & 0xFFFFu) + (key[i] >> 16);
                    if constexpr (RW == 2)
                        reinterpret_cast<uint2*>(sbuf)[q] = make_uint2(w[0], w[1]);
                    else
                        reinterpret_cast<uint4*>(sbuf)[q] = make_uint4(w[0], w[1], w[2], w[3]);
                    cellof[q] = static_cast<uint16_t>(cell);
                }
            }
            __syncthreads();
            if (sh_plan.simple)
                eval_sorted<D, O, true, TS>(sh_t, g, sh_plan, tile, org, cbase, sbuf, cellof, n, out, out_f32, C, ch);
            else
                eval_sorted_general<D, O, TS>(sh_t, g, sh_plan, tile, org, cbase, sbuf, cellof, n, out, out_f32, C,
                                              ch);
            __syncthreads();
        }
        }  // channel
        r = end;
    }
}

}  // namespace bin_detail
}  // namespace intp_gb300
