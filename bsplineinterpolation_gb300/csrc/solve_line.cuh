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
#include <type_traits>

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
};

// a * b + c with one rounding (FP32 or FP64).
__device__ __forceinline__ float fma_r(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_r(double a, double b, double c) { return __fma_rn(a, b, c); }

// Chunk accessors of one line: load(i0, cnt, buf) fills buf[0 .. cnt-1] with
// elements i0 .. i0+cnt-1 of the line, store(i0, cnt, buf) writes them back.

// Element k at base[k*S] (global memory; each lane its own line).
template <class R>
struct StridedChunks {
    R* base;
    int64_t S;
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
};

// A line held contiguously (in shared memory).
template <class R>
struct SmemChunks {
    R* base;
    template <int K>
    __device__ __forceinline__ void load(int64_t i0, int cnt, R (&buf)[K]) const {
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < cnt) buf[k] = base[i0 + k];
    }
    template <int K>
    __device__ __forceinline__ void store(int64_t i0, int cnt, const R (&buf)[K]) const {
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < cnt) base[i0 + k] = buf[k];
    }
};

// 32 consecutive contiguous lines, lane l owning line l0 + l (x = line l0's
// first element, `rows` lines present), each chunk moved through a per-warp
// [32][33] shared-memory transpose: the global accesses are runs of one
// line's elements (lane j touches element i0 + j of every line, all 32
// loads in flight), and lane l reading element k of its line touches bank
// (l + k) mod 32. Chunks are at most 32 elements. Warp-collective: every
// lane calls with the same chunk; lanes past `rows` compute on stale values
// that are never written back.
template <class R>
struct WarpContigChunks {
    R* x;
    int64_t n;
    int rows;
    R* stage;
    int lane;
    template <int K>
    __device__ __forceinline__ void load(int64_t i0, int cnt, R (&buf)[K]) const {
        static_assert(K <= 32, "chunks of at most 32 elements");
        __syncwarp();
        if (lane < cnt) {
            // rows in groups (32 FP32 / 16 FP64 loads in flight per lane)
            constexpr int G = sizeof(R) == 4 ? 32 : 16;
#pragma unroll
            for (int g = 0; g < 32; g += G) {
                R v[G];
#pragma unroll
                for (int r = 0; r < G; ++r)
                    if (g + r < rows) v[r] = x[(g + r) * n + i0 + lane];
#pragma unroll
                for (int r = 0; r < G; ++r) stage[(g + r) * 33 + lane] = v[r];
            }
        }
        __syncwarp();
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < cnt) buf[k] = stage[lane * 33 + k];
    }
    template <int K>
    __device__ __forceinline__ void store(int64_t i0, int cnt, const R (&buf)[K]) const {
        __syncwarp();
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < cnt) stage[lane * 33 + k] = buf[k];
        __syncwarp();
        if (lane < cnt) {
#pragma unroll
            for (int r = 0; r < 32; ++r)
                if (r < rows) x[r * n + i0 + lane] = stage[r * 33 + lane];
        }
    }
};

// WarpContigChunks for FP32 lines whose length is a multiple of 4 (every line
// starts 16-byte aligned): chunks of 16 elements move as float4 vectors
// through a per-warp [32][20] stage. Lane l = 4 * row_sub + q loads column
// group q (elements 4q .. 4q+3 of the chunk) of rows row_sub, +8, +16, +24;
// lane l then reads its own row as four float4 (16-byte units 5l + j: the
// eight lanes of a phase hit distinct bank groups). A chunk that does not
// start on a multiple of 4 (the cyclic corner read) takes per-element
// copies. Only data moves: results equal those of WarpContigChunks.
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

}  // namespace intp_gb300
