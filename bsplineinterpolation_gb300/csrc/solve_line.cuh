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

// Accessor of one line: element k at base[k*S].
template <class R>
struct StridedLine {
    R* base;
    int64_t S;
    __device__ __forceinline__ R load(int64_t k) const { return base[k * S]; }
    __device__ __forceinline__ void store(int64_t k, R v) const { base[k * S] = v; }
};

// A line held contiguously (in shared memory).
template <class R>
struct SmemLine {
    R* base;
    __device__ __forceinline__ R load(int64_t k) const { return base[k]; }
    __device__ __forceinline__ void store(int64_t k, R v) const { base[k] = v; }
};

template <class R, int P, int Q, bool CYC, class Line>
__device__ __forceinline__ void solve_line(const FactorView<R>& f, const Line& line) {
    const int64_t n = f.n;
    // ---- forward: y = L^{-1} x ----
    R win[P > 0 ? P : 1];  // y_{i-P} .. y_{i-1}
#pragma unroll
    for (int k = 0; k < P; ++k) win[k] = 0;
    R acc[Q > 0 ? Q : 1];  // cyclic: rows n-Q .. n-1 collecting side-band terms
    if (CYC) {
#pragma unroll
        for (int r = 0; r < Q; ++r) acc[r] = line.load(n - Q + r);
    }
    for (int64_t i = 0; i < n; ++i) {
        R v;
        if (CYC && i >= n - Q) {
            v = acc[0];
#pragma unroll
            for (int r = 1; r < Q; ++r)
                if (i == n - Q + r) v = acc[r];
        } else {
            v = line.load(i);
        }
#pragma unroll
        for (int k = 0; k < P; ++k) v -= __ldg(f.lower + i * P + k) * win[k];
        if (CYC && i < n - P - 1) {
#pragma unroll
            for (int r = 0; r < Q; ++r) acc[r] -= __ldg(f.bottom + r * n + i) * v;
        }
        line.store(i, v);
#pragma unroll
        for (int k = 0; k + 1 < P; ++k) win[k] = win[k + 1];
        if (P > 0) win[P - 1] = v;
    }
    // ---- back: x = U^{-1} y ----
    R zw[Q > 0 ? Q : 1];  // z_{i+1} .. z_{i+Q}
#pragma unroll
    for (int k = 0; k < Q; ++k) zw[k] = 0;
    R tail[P > 0 ? P : 1];  // cyclic: z_{n-P} .. z_{n-1}
#pragma unroll
    for (int k = 0; k < P; ++k) tail[k] = 0;
    for (int64_t i = n - 1; i >= 0; --i) {
        R v = line.load(i);
        if (CYC) {
#pragma unroll
            for (int r = P - 1; r >= 0; --r)
                if (n - P + r > i + Q) v -= __ldg(f.right + r * n + i) * tail[r];
        }
#pragma unroll
        for (int k = Q - 1; k >= 0; --k) v -= __ldg(f.upper + i * Q + k) * zw[k];
        v *= __ldg(f.dinv + i);
        line.store(i, v);
        if (CYC) {
#pragma unroll
            for (int r = 0; r < P; ++r)
                if (i == n - P + r) tail[r] = v;
        }
#pragma unroll
        for (int k = Q - 1; k > 0; --k) zw[k] = zw[k - 1];
        if (Q > 0) zw[0] = v;
    }
}

}  // namespace intp_gb300
