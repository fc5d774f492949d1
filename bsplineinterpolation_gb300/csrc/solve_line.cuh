// Band / cyclic-band substitution of one mesh line with a precomputed factor
// (BandLU.hpp:120-143 and :215-259), shared by the single-table solves
// (solve_kernels.cu) and the batched solves (batch.cu) so both round
// identically.
//
// Substitution order follows the reference's push loops restated as pulls:
// row i of the forward sweep subtracts L(i, i-p) .. L(i, i-1) in that order,
// the cyclic bottom rows first collect their side-band terms in increasing
// column order, and row i of the back sweep subtracts the right side band
// (columns n-1 down to n-p) before the main band (columns i+q down to i+1).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <climits>
#include <type_traits>

#include "dw.cuh"

namespace intp_gb300 {

template <class R>
struct FactorView {
    int64_t n;
    const R* lower;   // [n*P]
    const R* upper;   // [n*Q]
    const R* dinv;    // [n]
    const R* bottom;  // [Q*n]
    const R* right;   // [P*n]
    // rows clo .. chi-1 are identical to row clo: the substitution takes them
    // from registers (same values, no loads); clo = chi: none
    int64_t clo = 0, chi = 0;
    // cyclic: the bottom side-band entries of rows zside .. n-P-2 are all
    // zero (INT64_MAX: not known)
    int64_t zside = INT64_MAX;
};

// a * b + c with one rounding (FP32 or FP64).
__device__ __forceinline__ float fma_r(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_r(double a, double b, double c) { return __fma_rn(a, b, c); }

// Chunk accessors of one line: load(i0, cnt, buf) fills buf[0 .. cnt-1] with
// elements i0 .. i0+cnt-1 of the line, store(i0, cnt, buf) writes them back.
// An accessor with kPrefetch also moves chunks in two steps, so that the
// next chunk's loads are in flight while the current one is computed:
// fetch(i0, cnt, pend, slot) issues the loads, take(i0, cnt, pend, slot, buf)
// completes them into buf, and store(i0, cnt, buf, slot) writes back a chunk
// taken from `slot` (slots alternate between consecutive chunks).

// Element k at base[k*S] (global memory; each lane its own line).
// Prefetch: the next chunk's loads land in registers (Pending).
template <class R>
struct StridedChunks {
    R* base;
    int64_t S;
    static constexpr bool kPrefetch = true;
    template <int K>
    struct Pending {
        R v[K];
    };
    template <int K>
    __device__ __forceinline__ void load(int64_t i0, int cnt, R (&buf)[K]) const {
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < cnt) buf[k] = base[(i0 + k) * S];
    }
    template <int K>
    __device__ __forceinline__ void store(int64_t i0, int cnt, const R (&buf)[K]) const {
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < cnt) base[(i0 + k) * S] = buf[k];
    }
    template <int K>
    __device__ __forceinline__ void fetch(int64_t i0, int cnt, Pending<K>& p, int) const {
        load(i0, cnt, p.v);
    }
    template <int K>
    __device__ __forceinline__ void take(int64_t, int cnt, Pending<K>& p, int, R (&buf)[K]) const {
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < cnt) buf[k] = p.v[k];
    }
    template <int K>
    __device__ __forceinline__ void store(int64_t i0, int cnt, const R (&buf)[K], int) const {
        store(i0, cnt, buf);
    }
};

// One asynchronous global -> shared copy of BYTES (4 or 8) bytes.
template <int BYTES>
__device__ __forceinline__ void line_cp_async(void* dst_smem, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(
                     static_cast<uint32_t>(__cvta_generic_to_shared(dst_smem))),
                 "l"(src), "n"(BYTES)
                 : "memory");
}

// 32 consecutive contiguous lines, lane l owning line l0 + l (x = line l0's
// first element, `rows` lines present), each chunk moved through a per-warp
// shared-memory stage of [32][K+1] elements: the global accesses are runs of
// K elements of 32 / K lines per instruction (lane j touches element
// i0 + j % K of lines j / K, j / K + 32 / K, ...), and
// lane l reading element k of its line touches word l * (K+1) + k, distinct
// banks across the warp. Two stages (`stage` holds both, 2 * 32 * (K+1))
// alternate between consecutive chunks: a chunk's rows move into its slot's
// stage by cp.async (8- or 4-byte copies), in flight while the previous
// chunk is computed. Warp-collective: every lane calls with the same chunk;
// lanes past `rows` compute on stale values that are never written back.
template <class R, int K>
struct WarpContigChunksPF {
    R* x;
    int64_t n;
    int rows;
    R* stage;
    int lane;
    static constexpr bool kPrefetch = true;
    static constexpr int kPitch = K + 1;
    static constexpr int kStageElems = 2 * 32 * kPitch;
    template <int KK>
    struct Pending {};
    __device__ __forceinline__ R* slot_stage(int slot) const { return stage + slot * 32 * kPitch; }
    __device__ __forceinline__ void fetch(int64_t i0, int cnt, Pending<K>&, int slot) const {
        static_assert(sizeof(R) == 4 || sizeof(R) == 8, "4- or 8-byte elements");
        __syncwarp();  // the slot's previous chunk has been read out by every lane
        R* st = slot_stage(slot);
        // all lanes copy: lane l takes element l % K of rows l / K, + 32 / K, ...
        static_assert(32 % K == 0, "chunks of a power-of-two length up to 32");
        const int e = lane % K;
        if (e < cnt) {
            const R* src = x + i0 + e;
            for (int r = lane / K; r < rows; r += 32 / K) line_cp_async<sizeof(R)>(st + r * kPitch + e, src + r * n);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    __device__ __forceinline__ void take(int64_t, int cnt, Pending<K>&, int slot, R (&buf)[K]) const {
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncwarp();
        const R* st = slot_stage(slot);
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < cnt) buf[k] = st[lane * kPitch + k];
    }
    __device__ __forceinline__ void store(int64_t i0, int cnt, const R (&buf)[K], int slot) const {
        R* st = slot_stage(slot);
        __syncwarp();
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < cnt) st[lane * kPitch + k] = buf[k];
        __syncwarp();
        const int e = lane % K;
        if (e < cnt) {
            for (int r = lane / K; r < rows; r += 32 / K) x[r * n + i0 + e] = st[r * kPitch + e];
        }
    }
    // one-off chunks (the cyclic corner rows), through slot 0
    __device__ __forceinline__ void load(int64_t i0, int cnt, R (&buf)[K]) const {
        Pending<K> p;
        fetch(i0, cnt, p, 0);
        take(i0, cnt, p, 0, buf);
    }
    __device__ __forceinline__ void store(int64_t i0, int cnt, const R (&buf)[K]) const { store(i0, cnt, buf, 0); }
};

// Contiguous FP32 lines whose length is a multiple of 4 (every line
// starts 16-byte aligned): chunks of 16 elements move as float4 vectors
// through a per-warp [32][20] stage. Lane l = 4 * row_sub + q loads column
// group q (elements 4q .. 4q+3 of the chunk) of rows row_sub, +8, +16, +24;
// lane l then reads its own row as four float4 (16-byte units 5l + j: the
// eight lanes of a phase hit distinct bank groups). A chunk that does not
// start on a multiple of 4 (the cyclic corner read) takes per-element
// copies. Only data moves: results equal those of WarpContigChunksPF.
struct WarpContigChunksV4 {
    float* x;  // first element of line l0
    int64_t n;
    int rows;
    float* stage;  // 32 * 20 floats
    int lane;
    static constexpr int kPitch = 20;
    template <int K>
    __device__ __forceinline__ void load(int64_t i0, int cnt, float (&buf)[K]) const {
        static_assert(K <= 16, "chunks of at most 16 elements");
        __syncwarp();
        const int q = lane & 3;
        const bool vec = (i0 & 3) == 0;
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            const int r = (lane >> 2) + 8 * g;
            if (r < rows && 4 * q < cnt) {
                const float* src = x + r * n + i0 + 4 * q;
                float4 v;
                if (vec && 4 * q + 4 <= cnt) {
                    v = *reinterpret_cast<const float4*>(src);
                } else {
                    v.x = src[0];
                    v.y = 4 * q + 1 < cnt ? src[1] : 0.0f;
                    v.z = 4 * q + 2 < cnt ? src[2] : 0.0f;
                    v.w = 4 * q + 3 < cnt ? src[3] : 0.0f;
                }
                *reinterpret_cast<float4*>(stage + r * kPitch + 4 * q) = v;
            }
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < (K + 3) / 4; ++j) {
            const float4 v = *reinterpret_cast<const float4*>(stage + lane * kPitch + 4 * j);
            if (4 * j < K) buf[4 * j] = v.x;
            if (4 * j + 1 < K) buf[4 * j + 1] = v.y;
            if (4 * j + 2 < K) buf[4 * j + 2] = v.z;
            if (4 * j + 3 < K) buf[4 * j + 3] = v.w;
        }
    }
    template <int K>
    __device__ __forceinline__ void store(int64_t i0, int cnt, const float (&buf)[K]) const {
        static_assert(K <= 16, "chunks of at most 16 elements");
        __syncwarp();
#pragma unroll
        for (int j = 0; j < (K + 3) / 4; ++j) {
            float4 v;
            v.x = 4 * j < K ? buf[4 * j] : 0.0f;
            v.y = 4 * j + 1 < K ? buf[4 * j + 1] : 0.0f;
            v.z = 4 * j + 2 < K ? buf[4 * j + 2] : 0.0f;
            v.w = 4 * j + 3 < K ? buf[4 * j + 3] : 0.0f;
            *reinterpret_cast<float4*>(stage + lane * kPitch + 4 * j) = v;
        }
        __syncwarp();
        const int q = lane & 3;
        const bool vec = (i0 & 3) == 0;
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            const int r = (lane >> 2) + 8 * g;
            if (r < rows && 4 * q < cnt) {
                float* dst = x + r * n + i0 + 4 * q;
                const float4 v = *reinterpret_cast<const float4*>(stage + r * kPitch + 4 * q);
                if (vec && 4 * q + 4 <= cnt) {
                    *reinterpret_cast<float4*>(dst) = v;
                } else {
                    dst[0] = v.x;
                    if (4 * q + 1 < cnt) dst[1] = v.y;
                    if (4 * q + 2 < cnt) dst[2] = v.z;
                    if (4 * q + 3 < cnt) dst[3] = v.w;
                }
            }
        }
    }
};

// Substitution of one line with the band / cyclic-band factor, walking the
// line in chunks of K elements (K loads in flight per lane, the values of a
// chunk held in registers). Every step is the same sequence of roundings as
// the textbook recurrences written out with explicit FMAs, so all callers
// (strided lines, transposed contiguous lines, batched items) agree bit for
// bit.
// CONST_ROWS: take the factor's constant interior rows (FactorView::clo ..
// chi) from registers. It pays where one lane walks a long line alone (the
// factor loads of each chunk would wait on L2); where a warp's lanes share
// the factor row, the loads are broadcasts and the registers cost occupancy.
template <class Io, class = void>
struct chunks_prefetch : std::false_type {};
template <class Io>
struct chunks_prefetch<Io, std::void_t<decltype(Io::kPrefetch)>> : std::integral_constant<bool, Io::kPrefetch> {};

template <class R, int P, int Q, bool CYC, int K, class Io, bool CONST_ROWS = false>
__device__ __forceinline__ void solve_line_chunked(const FactorView<R>& f, const Io& io) {
    const int64_t n = f.n;
    // the factor's constant interior row, in registers (non-cyclic factors);
    // a chunk that lies inside [clo, chi) reads its rows from here
    const bool has_const = CONST_ROWS && !CYC && f.chi > f.clo;
    R cl[CONST_ROWS && P > 0 ? P : 1], cu[CONST_ROWS && Q > 0 ? Q : 1], cd = 0;
    if (has_const) {
#pragma unroll
        for (int kk = 0; kk < P; ++kk) cl[kk] = __ldg(f.lower + f.clo * P + kk);
#pragma unroll
        for (int kk = 0; kk < Q; ++kk) cu[kk] = __ldg(f.upper + f.clo * Q + kk);
        cd = __ldg(f.dinv + f.clo);
    }
    // ---- forward: y = L^{-1} x ----
    R win[P > 0 ? P : 1];  // y_{i-P} .. y_{i-1}
#pragma unroll
    for (int k = 0; k < P; ++k) win[k] = 0;
    R acc[Q > 0 ? Q : 1];  // cyclic: rows n-Q .. n-1 collecting side-band terms
    if (CYC) {
        R tmp[K];
        io.load(n - Q, Q, tmp);
#pragma unroll
        for (int r = 0; r < Q; ++r) acc[r] = tmp[r];
    }
    // one chunk's forward rows; CST: every row of the chunk is the constant row
    auto forward = [&](auto cst, int64_t i0, int cnt, R (&buf)[K]) {
        constexpr bool CST = decltype(cst)::value;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (k < cnt) {
                const int64_t i = i0 + k;
                R v = buf[k];
                if (CYC && i >= n - Q) {
                    v = acc[0];
#pragma unroll
                    for (int r = 1; r < Q; ++r)
                        if (i == n - Q + r) v = acc[r];
                }
#pragma unroll
                for (int kk = 0; kk < P; ++kk)
                    v = fma_r(-(CST ? cl[kk] : __ldg(f.lower + i * P + kk)), win[kk], v);
                if (CYC && i < n - P - 1) {
#pragma unroll
                    for (int r = 0; r < Q; ++r) acc[r] = fma_r(-__ldg(f.bottom + r * n + i), v, acc[r]);
                }
                buf[k] = v;
#pragma unroll
                for (int kk = 0; kk + 1 < P; ++kk) win[kk] = win[kk + 1];
                if (P > 0) win[P - 1] = v;
            }
        }
    };
    if constexpr (chunks_prefetch<Io>::value && !CONST_ROWS) {
        // the next chunk's loads are issued before this chunk is computed
        typename Io::template Pending<K> pend;
        int slot = 0;
        int cnt = static_cast<int>(n < K ? n : K);
        if (n > 0) io.fetch(0, cnt, pend, slot);
        for (int64_t i0 = 0; i0 < n; i0 += K) {
            R buf[K];
            io.take(i0, cnt, pend, slot, buf);
            const int64_t j0 = i0 + K;
            const int ncnt = static_cast<int>(j0 < n ? (n - j0 < K ? n - j0 : K) : 0);
            if (ncnt > 0) io.fetch(j0, ncnt, pend, slot ^ 1);
            forward(std::false_type{}, i0, cnt, buf);
            io.store(i0, cnt, buf, slot);
            slot ^= 1;
            cnt = ncnt;
        }
    } else {
        for (int64_t i0 = 0; i0 < n; i0 += K) {
            const int cnt = static_cast<int>(n - i0 < K ? n - i0 : K);
            R buf[K];
            io.load(i0, cnt, buf);
            if constexpr (CONST_ROWS) {
                if (has_const && i0 >= f.clo && i0 + cnt <= f.chi) {
                    forward(std::true_type{}, i0, cnt, buf);
                    io.store(i0, cnt, buf);
                    continue;
                }
            }
            forward(std::false_type{}, i0, cnt, buf);
            io.store(i0, cnt, buf);
        }
    }
    // ---- back: x = U^{-1} y ----
    R zw[Q > 0 ? Q : 1];  // z_{i+1} .. z_{i+Q}
#pragma unroll
    for (int k = 0; k < Q; ++k) zw[k] = 0;
    R tail[P > 0 ? P : 1];  // cyclic: z_{n-P} .. z_{n-1}
#pragma unroll
    for (int k = 0; k < P; ++k) tail[k] = 0;
    auto back = [&](auto cst, int64_t i0, int cnt, R (&buf)[K]) {
        constexpr bool CST = decltype(cst)::value;
#pragma unroll
        for (int k = K - 1; k >= 0; --k) {
            if (k < cnt) {
                const int64_t i = i0 + k;
                R v = buf[k];
                if (CYC) {
#pragma unroll
                    for (int r = P - 1; r >= 0; --r)
                        if (n - P + r > i + Q) v = fma_r(-__ldg(f.right + r * n + i), tail[r], v);
                }
#pragma unroll
                for (int kk = Q - 1; kk >= 0; --kk)
                    v = fma_r(-(CST ? cu[kk] : __ldg(f.upper + i * Q + kk)), zw[kk], v);
                v *= CST ? cd : __ldg(f.dinv + i);
                buf[k] = v;
                if (CYC) {
#pragma unroll
                    for (int r = 0; r < P; ++r)
                        if (i == n - P + r) tail[r] = v;
                }
#pragma unroll
                for (int kk = Q - 1; kk > 0; --kk) zw[kk] = zw[kk - 1];
                if (Q > 0) zw[0] = v;
            }
        }
    };
    if constexpr (chunks_prefetch<Io>::value && !CONST_ROWS) {
        // the forward sweep's stores (other lanes' too) before the first
        // asynchronous read of this sweep
        __threadfence_block();
        typename Io::template Pending<K> pend;
        int slot = 0;
        int cnt = static_cast<int>(n < K ? n : K);
        if (n > 0) io.fetch(n - cnt, cnt, pend, slot);
        for (int64_t i1 = n - 1; i1 >= 0; i1 -= K) {
            const int64_t i0 = i1 - cnt + 1;
            R buf[K];
            io.take(i0, cnt, pend, slot, buf);
            const int ncnt = static_cast<int>(i0 < K ? i0 : K);
            if (ncnt > 0) io.fetch(i0 - ncnt, ncnt, pend, slot ^ 1);
            back(std::false_type{}, i0, cnt, buf);
            io.store(i0, cnt, buf, slot);
            slot ^= 1;
            cnt = ncnt;
        }
    } else {
        for (int64_t i1 = n - 1; i1 >= 0; i1 -= K) {
            const int cnt = static_cast<int>(i1 + 1 < K ? i1 + 1 : K);
            const int64_t i0 = i1 - cnt + 1;
            R buf[K];
            io.load(i0, cnt, buf);
            if constexpr (CONST_ROWS) {
                if (has_const && i0 >= f.clo && i0 + cnt <= f.chi) {
                    back(std::true_type{}, i0, cnt, buf);
                    io.store(i0, cnt, buf);
                    continue;
                }
            }
            back(std::false_type{}, i0, cnt, buf);
            io.store(i0, cnt, buf);
        }
    }
}

// ---------------------------------------------------------------------------
// Warp-segmented substitution of one line (all 32 lanes of a warp call).
//
// Each sweep's rows are cut into 32 segments, one per lane. A lane runs the
// recurrence over the W rows before its segment from a zero state, then over
// its segment, writing it. The zero state's error decays geometrically (the
// factor's recurrences are contractions for B-spline collocation: about
// 0.27 per row at order 3, 0.6 at order 7), and once P consecutive values
// equal the serial sweep's bit for bit, every later value does too (the
// same operations on the same operands). A lane then checks exactly that:
// its warm-up values at the P rows before its segment against the values
// its neighbour wrote there. A lane whose check fails is recomputed from
// its neighbour's (exact) values, lowest lane first, and the next lane is
// checked again. The result therefore equals the serial sweep's
// (solve_line_chunked) bit for bit, whatever W is; W only sets how rarely a
// segment is recomputed (64 rows in FP32 and 128 in FP64 lock every order;
// a host simulation of orders 1..7 locked within 47 rows in FP32).
//
// Cyclic factors: the forward segments cover rows 0 .. n-Q-1; the bottom
// rows' side-band sums are then formed by one lane in row order over the
// rows with nonzero side-band entries (FactorView::zside onwards they are
// +0, whose products leave a finite nonzero sum unchanged; where that does
// not hold, the whole row range is walked), and the last Q rows follow
// serially. The back sweep first computes the last P rows serially (their
// values are the side-band operands of every other row), then the
// segments cover rows 0 .. n-P-1.
// ---------------------------------------------------------------------------

// Test hook (one copy per translation unit): when >= 0, solve_line_warp
// warms up over at most this many rows, so that its recompute path runs.
static __device__ int g_warm_rows_cap = -1;

#define INTP_DEFINE_WARM_CAP_SETTER(NAME)                                                     \
    cudaError_t NAME(int rows) {                                                               \
        return cudaMemcpyToSymbol(g_warm_rows_cap, &rows, sizeof(int), 0, cudaMemcpyHostToDevice); \
    }

template <class R>
__device__ __forceinline__ bool bits_equal(R a, R b) {
    if constexpr (std::is_same<R, DW>::value)
        return __float_as_uint(a.hi) == __float_as_uint(b.hi) && __float_as_uint(a.lo) == __float_as_uint(b.lo);
    else if constexpr (sizeof(R) == 4)
        return __float_as_uint(a) == __float_as_uint(b);
    else
        return __double_as_longlong(a) == __double_as_longlong(b);
}

// Element i of a line at base[i * S].
template <class R>
struct LineRef {
    R* base;
    int64_t S;
    __device__ __forceinline__ R ld(int64_t i) const { return base[i * S]; }
    __device__ __forceinline__ void st(int64_t i, R v) const { base[i * S] = v; }
};

// Factor rows of one line, from memory or (rows clo .. chi-1 with
// CONST_ROWS) from registers.
template <class R, int P, int Q, bool CYC, bool CONST_ROWS>
struct FactorRows {
    static constexpr int P1 = P > 0 ? P : 1, Q1 = Q > 0 ? Q : 1;
    const FactorView<R>& f;
    bool has_const;
    R cl[P1], cu[Q1], cd, cb[Q1], cr[P1];
    __device__ __forceinline__ explicit FactorRows(const FactorView<R>& fv) : f(fv), cd(0) {
        has_const = CONST_ROWS && f.chi > f.clo;
        if (has_const) {
#pragma unroll
            for (int kk = 0; kk < P; ++kk) cl[kk] = __ldg(f.lower + f.clo * P + kk);
#pragma unroll
            for (int kk = 0; kk < Q; ++kk) cu[kk] = __ldg(f.upper + f.clo * Q + kk);
            cd = __ldg(f.dinv + f.clo);
            if (CYC) {
#pragma unroll
                for (int r = 0; r < Q; ++r) cb[r] = __ldg(f.bottom + r * f.n + f.clo);
#pragma unroll
                for (int r = 0; r < P; ++r) cr[r] = __ldg(f.right + r * f.n + f.clo);
            }
        }
    }
    __device__ __forceinline__ bool in_const(int64_t i) const { return has_const && i >= f.clo && i < f.chi; }
    __device__ __forceinline__ void lower(int64_t i, R (&l)[P1]) const {
        const bool c = in_const(i);
#pragma unroll
        for (int kk = 0; kk < P; ++kk) l[kk] = c ? cl[kk] : __ldg(f.lower + i * P + kk);
    }
    __device__ __forceinline__ void upper(int64_t i, R (&u)[Q1], R& d, R (&rr)[P1]) const {
        const bool c = in_const(i);
#pragma unroll
        for (int kk = 0; kk < Q; ++kk) u[kk] = c ? cu[kk] : __ldg(f.upper + i * Q + kk);
        d = c ? cd : __ldg(f.dinv + i);
        if (CYC) {
#pragma unroll
            for (int r = 0; r < P; ++r) rr[r] = c ? cr[r] : __ldg(f.right + r * f.n + i);
        }
    }
};

// One forward row (without the cyclic side-band sums): v = x_i - L(i, i-P ..
// i-1) . win, in solve_line_chunked's order; win shifts in v.
template <class R, int P, int Q, bool CYC, bool CONST_ROWS>
__device__ __forceinline__ R forward_row(const FactorRows<R, P, Q, CYC, CONST_ROWS>& fr, int64_t i, R v,
                                         R (&win)[P > 0 ? P : 1]) {
    R l[P > 0 ? P : 1];
    fr.lower(i, l);
#pragma unroll
    for (int kk = 0; kk < P; ++kk) v = fma_r(-l[kk], win[kk], v);
#pragma unroll
    for (int kk = 0; kk + 1 < P; ++kk) win[kk] = win[kk + 1];
    if (P > 0) win[P - 1] = v;
    return v;
}

// One back row: the right side band against tail (cyclic), the band against
// zw, times dinv; zw shifts in the result.
template <class R, int P, int Q, bool CYC, bool CONST_ROWS>
__device__ __forceinline__ R back_row(const FactorRows<R, P, Q, CYC, CONST_ROWS>& fr, int64_t i, R v,
                                      R (&zw)[Q > 0 ? Q : 1], const R (&tail)[P > 0 ? P : 1]) {
    constexpr int P1 = P > 0 ? P : 1, Q1 = Q > 0 ? Q : 1;
    R u[Q1], d, rr[P1];
    fr.upper(i, u, d, rr);
    const int64_t n = fr.f.n;
    if (CYC) {
#pragma unroll
        for (int r = P - 1; r >= 0; --r)
            if (n - P + r > i + Q) v = fma_r(-rr[r], tail[r], v);
    }
#pragma unroll
    for (int kk = Q - 1; kk >= 0; --kk) v = fma_r(-u[kk], zw[kk], v);
    v *= d;
#pragma unroll
    for (int kk = Q - 1; kk > 0; --kk) zw[kk] = zw[kk - 1];
    if (Q > 0) zw[0] = v;
    return v;
}

template <class R, int N>
__device__ __forceinline__ bool states_equal(const R (&a)[N], const R (&b)[N], int count) {
    bool ok = true;
#pragma unroll
    for (int k = 0; k < N; ++k) ok = ok && (k >= count || bits_equal(a[k], b[k]));
    return ok;
}

template <class R, int P, int Q, bool CYC, int W, bool CONST_ROWS = false, class Line = LineRef<R>>
__device__ __forceinline__ void solve_line_warp(const FactorView<R>& f, const Line& x, int lane) {
    constexpr int P1 = P > 0 ? P : 1, Q1 = Q > 0 ? Q : 1;
    constexpr unsigned kAll = 0xffffffffu;
    const int64_t n = f.n;
    if (n <= 0) return;
    const FactorRows<R, P, Q, CYC, CONST_ROWS> fr(f);
    int64_t Wr = W;
    {
        const int cap = g_warm_rows_cap;
        if (cap >= 0 && cap < W) Wr = cap;
    }
    // segment length: odd, so the 32 lanes' rows of one step fall in
    // distinct shared-memory banks
    auto seg_len = [](int64_t m) {
        const int64_t L = (m + 31) / 32;
        return L | 1;
    };

    // ---- forward: rows 0 .. nf-1 in segments ----
    // Phase A: warm-up and segment without stores, giving the state entering
    // the segment (start) and the state leaving it (end). Lane order fixes
    // the starts: lane 0 and any lane whose warm-up began at row 0 start
    // exactly; a later lane's start is exact when it equals, bit for bit,
    // its (exact) predecessor's end, and is replaced by that end otherwise.
    // Phase B: every lane runs its segment from its start, storing it.
    const int64_t nf = CYC ? n - Q : n;
    {
        const int64_t L = seg_len(nf);
        const int64_t a = lane * L < nf ? lane * L : nf, b = a + L < nf ? a + L : nf;
        const int64_t s0 = a - Wr > 0 ? a - Wr : 0;
        R start[P1], end[P1];
#pragma unroll
        for (int k = 0; k < P1; ++k) start[k] = 0;
#pragma unroll 4
        for (int64_t i = s0; i < a; ++i) forward_row(fr, i, x.ld(i), start);
        auto run = [&]() {
#pragma unroll
            for (int k = 0; k < P1; ++k) end[k] = start[k];
#pragma unroll 4
            for (int64_t i = a; i < b; ++i) forward_row(fr, i, x.ld(i), end);
        };
        run();
        auto mismatch = [&]() {
            R prev[P1];
#pragma unroll
            for (int k = 0; k < P1; ++k) prev[k] = __shfl_up_sync(kAll, end[k], 1);
            return s0 > 0 && a < b && !states_equal(start, prev, P);
        };
        unsigned bad = __ballot_sync(kAll, mismatch());
        while (bad) {
            const int fl = __ffs(bad) - 1;
            R prev[P1];
#pragma unroll
            for (int k = 0; k < P1; ++k) prev[k] = __shfl_sync(kAll, end[k], fl > 0 ? fl - 1 : 0);
            if (lane == fl) {
#pragma unroll
                for (int k = 0; k < P1; ++k) start[k] = prev[k];
                run();
            }
            bad &= ~(1u << fl);
            const bool m = mismatch();
            const unsigned again = __ballot_sync(kAll, lane == fl + 1 && m);
            bad = (bad & ~(2u << fl)) | again;
        }
        {
            R win[P1];
#pragma unroll
            for (int k = 0; k < P1; ++k) win[k] = start[k];
#pragma unroll 4
            for (int64_t i = a; i < b; ++i) x.st(i, forward_row(fr, i, x.ld(i), win));
        }
        __syncwarp();
    }
    if (CYC) {
        // the bottom rows' side-band sums in row order, then rows n-Q .. n-1
        const int64_t nb = n - P - 1;  // rows feeding the sums: 0 .. nb-1
        const int64_t z = f.zside < nb ? f.zside : nb;
        // the +0 entries of rows z .. nb-1 leave a sum unchanged unless the
        // sum is 0 or not finite, or a row value is not finite
        bool odd = false;
        for (int64_t i = z + lane; i < nb; i += 32) {
            const R v = x.ld(i);
            odd = odd || !(v - v == R(0));
        }
        odd = __any_sync(kAll, odd);
        if (lane == 0) {
            R acc[Q1];
#pragma unroll
            for (int r = 0; r < Q; ++r) acc[r] = x.ld(n - Q + r);
            for (int64_t i = 0; i < z; ++i) {
                const R v = x.ld(i);
#pragma unroll
                for (int r = 0; r < Q; ++r) acc[r] = fma_r(-__ldg(f.bottom + r * n + i), v, acc[r]);
            }
#pragma unroll
            for (int r = 0; r < Q; ++r) odd = odd || !(acc[r] != R(0) && acc[r] - acc[r] == R(0));
            if (odd) {
                for (int64_t i = z; i < nb; ++i) {
                    const R v = x.ld(i);
#pragma unroll
                    for (int r = 0; r < Q; ++r) acc[r] = fma_r(-__ldg(f.bottom + r * n + i), v, acc[r]);
                }
            }
            R win[P1];
#pragma unroll
            for (int k = 0; k < P1; ++k) win[k] = 0;
#pragma unroll
            for (int k = 0; k < P; ++k)
                if (nf - P + k >= 0) win[k] = x.ld(nf - P + k);
#pragma unroll
            for (int r = 0; r < Q; ++r) x.st(nf + r, forward_row(fr, nf + r, acc[r], win));
        }
        __syncwarp();
    }

    // ---- back: rows nk-1 .. 0 in segments, the same two phases from the
    // top lane down ----
    R tail[P1];  // cyclic: x_{n-P} .. x_{n-1}
#pragma unroll
    for (int k = 0; k < P1; ++k) tail[k] = 0;
    R top[Q1];  // the state entering row nk-1 from above
#pragma unroll
    for (int k = 0; k < Q1; ++k) top[k] = 0;
    const int64_t nk = CYC ? n - P : n;
    if (CYC) {
        if (lane == 0) {
            R zw[Q1];
#pragma unroll
            for (int k = 0; k < Q1; ++k) zw[k] = 0;
            for (int64_t i = n - 1; i >= nk; --i) x.st(i, back_row(fr, i, x.ld(i), zw, tail));
        }
        __syncwarp();
#pragma unroll
        for (int r = 0; r < P; ++r) tail[r] = x.ld(n - P + r);
#pragma unroll
        for (int kk = 0; kk < Q; ++kk) top[kk] = x.ld(nk + kk);
    }
    {
        const int64_t L = seg_len(nk);
        const int64_t a = lane * L < nk ? lane * L : nk, b = a + L < nk ? a + L : nk;
        const int64_t t0 = b + Wr < nk ? b + Wr : nk;  // warm-up rows b .. t0-1
        R start[Q1], end[Q1];
#pragma unroll
        for (int k = 0; k < Q1; ++k) start[k] = t0 == nk ? top[k] : R(0);
#pragma unroll 4
        for (int64_t i = t0 - 1; i >= b; --i) back_row(fr, i, x.ld(i), start, tail);
        auto run = [&]() {
#pragma unroll
            for (int k = 0; k < Q1; ++k) end[k] = start[k];
#pragma unroll 4
            for (int64_t i = b - 1; i >= a; --i) back_row(fr, i, x.ld(i), end, tail);
        };
        run();
        auto mismatch = [&]() {
            R next[Q1];
#pragma unroll
            for (int k = 0; k < Q1; ++k) next[k] = __shfl_down_sync(kAll, end[k], 1);
            return t0 < nk && a < b && !states_equal(start, next, Q);
        };
        unsigned bad = __ballot_sync(kAll, mismatch());
        while (bad) {
            const int fl = 31 - __clz(bad);
            R next[Q1];
#pragma unroll
            for (int k = 0; k < Q1; ++k) next[k] = __shfl_sync(kAll, end[k], fl < 31 ? fl + 1 : 31);
            if (lane == fl) {
#pragma unroll
                for (int k = 0; k < Q1; ++k) start[k] = next[k];
                run();
            }
            bad &= ~(1u << fl);
            const bool m = mismatch();
            const unsigned again = __ballot_sync(kAll, lane == fl - 1 && m);
            bad = (bad & ~(fl > 0 ? 1u << (fl - 1) : 0u)) | again;
        }
        {
            R zw[Q1];
#pragma unroll
            for (int k = 0; k < Q1; ++k) zw[k] = start[k];
#pragma unroll 4
            for (int64_t i = b - 1; i >= a; --i) x.st(i, back_row(fr, i, x.ld(i), zw, tail));
        }
    }
}

}  // namespace intp_gb300
