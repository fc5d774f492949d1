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

#include "async_copy.cuh"

namespace intp_gb300 {

template <class R>
struct FactorView {
    int64_t n;
    const R* lower;   // [n*P]
    const R* upper;   // [n*Q]
    const R* dinv;    // [n]
    const R* bottom;  // [Q*n]
    const R* right;   // [P*n]
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

// StridedChunks with the chunk loads streamed ahead through shared memory:
// each thread keeps a ring of NB chunk buffers (cp.async element copies, one
// commit group per chunk) and, when the substitution asks for chunk c, the
// copies of chunks c+1 .. c+NB-1 are already in flight. The loaded values
// and the arithmetic are those of StridedChunks; only the waiting changes
// (the serial chain of a line no longer waits a memory latency per chunk)
// and no registers hold data in flight.
//
// The substitution's request order is fixed: (cyclic only) the last Q
// elements, the forward chunks i0 = 0, K, 2K, ..., then the back chunks
// ending at n-1, n-1-K, .... The ring follows that order; the back chunks
// are fetched only after the forward sweep has written the whole line (a
// block fence orders those writes before the copies that read them back).
// ring[slot][k][tid]: thread-fastest, so a warp's accesses to one buffer
// element are conflict-free.
template <class R, int K, int NB>
struct PrefetchStridedChunks {
    R* base;
    int64_t S;
    int64_t n;
    R* ring;       // NB * K * nthreads elements
    int nthreads;
    int tid;
    bool cyc_head;  // the cyclic substitution's first request (last Q elements) comes first
    int Q;
    // request sequence state
    mutable int next_req;    // index of the next request in the forward+back order
    mutable int next_issue;  // index of the next chunk to issue
    int nf;                  // forward chunks
    __device__ __forceinline__ int total() const { return 2 * nf; }
    // chunk j of the sequence: [lo, lo + cnt)
    __device__ __forceinline__ void chunk(int j, int64_t& lo, int& cnt) const {
        if (j < nf) {
            lo = static_cast<int64_t>(j) * K;
            cnt = static_cast<int>(n - lo < K ? n - lo : K);
        } else {
            const int64_t i1 = n - 1 - static_cast<int64_t>(j - nf) * K;
            cnt = static_cast<int>(i1 + 1 < K ? i1 + 1 : K);
            lo = i1 - cnt + 1;
        }
    }
    __device__ __forceinline__ R* slot(int j, int k) const { return ring + ((j % NB) * K + k) * nthreads + tid; }
    __device__ __forceinline__ void issue(int j) const {
        int64_t lo;
        int cnt;
        chunk(j, lo, cnt);
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < cnt) cp_async<sizeof(R)>(slot(j, k), base + (lo + k) * S);
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    // issue chunks up to `upto` (exclusive), forward chunks any time, back
    // chunks once the forward sweep is done (next_req >= nf)
    __device__ __forceinline__ void fill(int upto) const {
        while (next_issue < upto && next_issue < total()) {
            if (next_issue >= nf && next_req < nf) break;
            issue(next_issue++);
        }
    }
    template <int KK>
    __device__ __forceinline__ void load(int64_t i0, int cnt, R (&buf)[KK]) const {
        static_assert(KK == K, "chunk size of the ring");
        if (cyc_head && next_req < 0) {
            // the cyclic head: a direct load of the last Q elements
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (k < cnt) buf[k] = base[(i0 + k) * S];
            next_req = 0;
            return;
        }
        if (next_req == nf) __threadfence_block();  // the forward writes before the back copies
        fill(next_req + NB);
        // wait for chunk next_req: groups complete in order, and at most
        // next_issue - next_req - 1 later ones may stay pending
        const int pending = next_issue - next_req - 1;
        if (pending >= 2)
            asm volatile("cp.async.wait_group 2;" ::: "memory");
        else if (pending == 1)
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        else
            asm volatile("cp.async.wait_group 0;" ::: "memory");
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < cnt) buf[k] = *slot(next_req, k);
        ++next_req;
    }
    template <int KK>
    __device__ __forceinline__ void store(int64_t i0, int cnt, const R (&buf)[KK]) const {
#pragma unroll
        for (int k = 0; k < KK; ++k)
            if (k < cnt) base[(i0 + k) * S] = buf[k];
    }
};

// Substitution of one line with the band / cyclic-band factor, walking the
// line in chunks of K elements (K loads in flight per lane, the values of a
// chunk held in registers). Every step is the same sequence of roundings as
// the textbook recurrences written out with explicit FMAs, so all callers
// (strided lines, transposed contiguous lines, batched items) agree bit for
// bit.
template <class R, int P, int Q, bool CYC, int K, class Io>
__device__ __forceinline__ void solve_line_chunked(const FactorView<R>& f, const Io& io) {
    const int64_t n = f.n;
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
    for (int64_t i0 = 0; i0 < n; i0 += K) {
        const int cnt = static_cast<int>(n - i0 < K ? n - i0 : K);
        R buf[K];
        io.load(i0, cnt, buf);
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
                for (int kk = 0; kk < P; ++kk) v = fma_r(-__ldg(f.lower + i * P + kk), win[kk], v);
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
        io.store(i0, cnt, buf);
    }
    // ---- back: x = U^{-1} y ----
    R zw[Q > 0 ? Q : 1];  // z_{i+1} .. z_{i+Q}
#pragma unroll
    for (int k = 0; k < Q; ++k) zw[k] = 0;
    R tail[P > 0 ? P : 1];  // cyclic: z_{n-P} .. z_{n-1}
#pragma unroll
    for (int k = 0; k < P; ++k) tail[k] = 0;
    for (int64_t i1 = n - 1; i1 >= 0; i1 -= K) {
        const int cnt = static_cast<int>(i1 + 1 < K ? i1 + 1 : K);
        const int64_t i0 = i1 - cnt + 1;
        R buf[K];
        io.load(i0, cnt, buf);
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
                for (int kk = Q - 1; kk >= 0; --kk) v = fma_r(-__ldg(f.upper + i * Q + kk), zw[kk], v);
                v *= __ldg(f.dinv + i);
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
        io.store(i0, cnt, buf);
    }
}

}  // namespace intp_gb300
