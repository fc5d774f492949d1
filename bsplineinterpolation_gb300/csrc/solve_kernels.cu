// Control-point solve: per-axis band / cyclic-band substitution over every
// mesh line (InterpolationTemplate.hpp:448-580, BandLU.hpp:120-143 and
// :215-259), in FP64, FP32 and double-word arithmetic (the mixed form).
//
// A mesh of shape N_0 x ... x N_{D-1} is processed one axis at a time. Along
// axis a the lines are indexed by (outer o, inner t): element k of a line is
// at o*N_a*S + k*S + t with S = prod_{d>a} N_d. One thread owns one line and
// walks it in register chunks of 32 elements (forward sweep, then back
// sweep, each chunk written back in place); adjacent threads own adjacent
// t, so for S >= 32 every chunk access is coalesced. The contiguous axis
// (S = 1) moves each chunk through a small per-warp shared-memory transpose
// so it is read and written coalesced too. Nothing holds a whole line, so
// occupancy is set by registers and long lines need no special path. The
// reference instead rotates the whole tensor after each axis pass
// (:537-543); solving in place along strided lines needs no rotation. The
// substitution itself is solve_line_chunked (solve_line.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "async_copy.cuh"
#include "launch.hpp"
#include "solve_line.cuh"

namespace intp_gb300 {

namespace {

// 32-bit index math for up to 2^30 values (grid-stride sums stay in range).
constexpr int64_t kIndex32Max = int64_t{1} << 30;

int grid_for(int64_t n, int block, int max_blocks) {
    int64_t g = (n + block - 1) / block;
    if (g > max_blocks) g = max_blocks;
    if (g < 1) g = 1;
    return static_cast<int>(g);
}

// Lines are walked in chunks of elements held in registers: 16 FP32 or 8 FP64
// values per lane (register budget: one wave of line groups per pass at
// 256^3; longer chunks cost a second wave).
template <class R>
constexpr int line_chunk() {
    return sizeof(R) == 4 ? 16 : 8;
}
constexpr int kSolveWarps = 4;  // warps per block

// Lines of at least kWarpLineMin elements, fewer than kWarpLineMaxLines of
// them (under one line per lane on every SM), are solved a warp per line.
constexpr int64_t kWarpLineMin = 128;
constexpr int64_t kWarpLineMaxLines = 152 * 32;

// Warm-up rows of the warp-segmented substitution: enough for the zero
// state's error to fall below the last bit in FP32 / FP64.
template <class R>
constexpr int warm_rows() {
    return sizeof(R) == 4 ? 64 : 128;
}

// Strided axis (S > 1): one thread per line; adjacent threads own adjacent
// lines (adjacent t), so every chunk load and store of a warp is a run of
// contiguous elements. No shared memory: occupancy is set by registers only.
template <class R, int P, int Q, bool CYC>
__global__ void __launch_bounds__(kSolveWarps * 32, 4) solve_warp_strided_kernel(R* __restrict__ x, int64_t n,
                                                                              int64_t S, int64_t nlines,
                                                                              FactorView<R> f) {
    for (int64_t l = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; l < nlines;
         l += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t o = l / S, t = l - o * S;
        solve_line_chunked<R, P, Q, CYC, line_chunk<R>()>(f, StridedChunks<R>{x + o * n * S + t, S});
    }
}

// Contiguous axis (S = 1): one warp per 32 consecutive lines, each chunk's
// rows copied into a shared-memory stage while the previous chunk is solved.
template <class R, int P, int Q, bool CYC>
__global__ void __launch_bounds__(kSolveWarps * 32, 4) solve_warp_contig_kernel(R* __restrict__ x, int64_t n,
                                                                             int64_t nlines, FactorView<R> f) {
    using Io = WarpContigChunksPF<R, line_chunk<R>()>;
    __shared__ __align__(16) R stage[kSolveWarps][Io::kStageElems];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t ngroups = (nlines + 31) / 32;
    for (int64_t g = blockIdx.x * static_cast<int64_t>(kSolveWarps) + warp; g < ngroups;
         g += static_cast<int64_t>(gridDim.x) * kSolveWarps) {
        const int64_t l0 = g * 32;
        const int rows = static_cast<int>(nlines - l0 < 32 ? nlines - l0 : 32);
        Io io{x + l0 * n, n, rows, stage[warp], lane};
        solve_line_chunked<R, P, Q, CYC, line_chunk<R>()>(f, io);
    }
}

// Contiguous FP32 lines of a length divisible by 4, 16-byte aligned: the
// chunks move as float4 vectors (WarpContigChunksV4).
template <int P, int Q, bool CYC>
__global__ void __launch_bounds__(kSolveWarps * 32, 4) solve_warp_contig_v4_kernel(float* __restrict__ x, int64_t n,
                                                                                int64_t nlines,
                                                                                FactorView<float> f) {
    __shared__ __align__(16) float stage[kSolveWarps][32 * WarpContigChunksV4::kPitch];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t ngroups = (nlines + 31) / 32;
    for (int64_t g = blockIdx.x * static_cast<int64_t>(kSolveWarps) + warp; g < ngroups;
         g += static_cast<int64_t>(gridDim.x) * kSolveWarps) {
        const int64_t l0 = g * 32;
        const int rows = static_cast<int>(nlines - l0 < 32 ? nlines - l0 : 32);
        WarpContigChunksV4 io{x + l0 * n, n, rows, stage[warp], lane};
        solve_line_chunked<float, P, Q, CYC, line_chunk<float>()>(f, io);
    }
}

// Few long lines: one warp per line, the line cut into 32 segments
// (solve_line_warp; the same values as one lane walking it).
template <class R, int P, int Q, bool CYC>
__global__ void __launch_bounds__(kSolveWarps * 32) solve_warp_line_kernel(R* __restrict__ x, int64_t n, int64_t S,
                                                                           int64_t nlines, FactorView<R> f) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t l = blockIdx.x * static_cast<int64_t>(kSolveWarps) + warp; l < nlines;
         l += static_cast<int64_t>(gridDim.x) * kSolveWarps) {
        const int64_t o = l / S, t = l - o * S;
        solve_line_warp<R, P, Q, CYC, warm_rows<R>(), true>(f, LineRef<R>{x + o * n * S + t, S}, lane);
    }
}

template <class R, int P, int Q, bool CYC>
cudaError_t launch_solve_pq(R* x, int64_t n, int64_t S, int64_t nlines, const FactorView<R>& f,
                            cudaStream_t s) {
    constexpr int kThreads = kSolveWarps * 32;
    if (n >= kWarpLineMin && nlines < kWarpLineMaxLines) {
        const int grid = grid_for(nlines, kSolveWarps, 152 * 64);
        solve_warp_line_kernel<R, P, Q, CYC><<<grid, kThreads, 0, s>>>(x, n, S, nlines, f);
    } else if (S == 1) {
        const int64_t groups = (nlines + 31) / 32;
        const int grid = grid_for(groups, kSolveWarps, 152 * 64);
        bool vec = false;
        if constexpr (sizeof(R) == 4) vec = n % 4 == 0 && reinterpret_cast<uintptr_t>(x) % 16 == 0;
        if constexpr (sizeof(R) == 4) {
            if (vec) solve_warp_contig_v4_kernel<P, Q, CYC><<<grid, kThreads, 0, s>>>(x, n, nlines, f);
        }
        if (!vec) solve_warp_contig_kernel<R, P, Q, CYC><<<grid, kThreads, 0, s>>>(x, n, nlines, f);
    } else {
        const int grid = grid_for(nlines, kThreads, 152 * 64);
        solve_warp_strided_kernel<R, P, Q, CYC><<<grid, kThreads, 0, s>>>(x, n, S, nlines, f);
    }
    note_launch();
    return cudaGetLastError();
}

template <class R>
cudaError_t launch_solve_r(R* x, int64_t n, int64_t S, int64_t nlines, int p, int q, bool cyclic,
                           const FactorView<R>& f, cudaStream_t s) {
    if (p != q) return cudaErrorInvalidValue;
    if (cyclic) {
        switch (p) {
            case 0: return launch_solve_pq<R, 0, 0, true>(x, n, S, nlines, f, s);
            case 1: return launch_solve_pq<R, 1, 1, true>(x, n, S, nlines, f, s);
            case 2: return launch_solve_pq<R, 2, 2, true>(x, n, S, nlines, f, s);
            case 3: return launch_solve_pq<R, 3, 3, true>(x, n, S, nlines, f, s);
        }
        return cudaErrorInvalidValue;
    }
    switch (p) {
        case 0: return launch_solve_pq<R, 0, 0, false>(x, n, S, nlines, f, s);
        case 1: return launch_solve_pq<R, 1, 1, false>(x, n, S, nlines, f, s);
        case 2: return launch_solve_pq<R, 2, 2, false>(x, n, S, nlines, f, s);
        case 3: return launch_solve_pq<R, 3, 3, false>(x, n, S, nlines, f, s);
        case 4: return launch_solve_pq<R, 4, 4, false>(x, n, S, nlines, f, s);
        case 5: return launch_solve_pq<R, 5, 5, false>(x, n, S, nlines, f, s);
        case 6: return launch_solve_pq<R, 6, 6, false>(x, n, S, nlines, f, s);
    }
    return cudaErrorInvalidValue;
}

// ---- data movement and residual kernels ----

// dst[shift(i)] = (To) src[i]: periodic axes move index i to (i + O/2) mod n
// (InterpolationTemplate.hpp:451-462). With dlo (FP32 destination) the copy
// is the double-float split of the values, dst = high part (also written to
// dst2, the solve's working copy) and dlo = the remainder. `identity`: no
// axis is shifted and there is one channel (destination index = source
// index). I is the index type (32-bit when the table allows).
template <class To, class I>
__global__ void __launch_bounds__(256) shift_copy_kernel(const double* __restrict__ src, To* __restrict__ dst,
                                                         float* __restrict__ dlo, float* __restrict__ dst2,
                                                         ShiftDesc sd, int identity) {
    const I C = static_cast<I>(sd.channels), total = static_cast<I>(sd.total);
    const I N = total * C;
    for (I j = blockIdx.x * static_cast<I>(blockDim.x) + threadIdx.x; j < N;
         j += static_cast<I>(gridDim.x) * blockDim.x) {
        I o = j;
        if (!identity) {
            // source element j = point i, channel ch (channel fastest); the
            // destination holds channel ch's mesh at ch * total
            const I i = C == 1 ? j : j / C, ch = j - i * C;
            I r = i;
            o = ch * total;
#pragma unroll
            for (int d = 3; d >= 0; --d) {
                if (d < sd.dim) {
                    const I n = static_cast<I>(sd.n[d]);
                    const I q = r / n;
                    I idx = r - q * n;
                    r = q;
                    if (sd.shift[d]) {
                        idx += static_cast<I>(sd.shift[d]);
                        if (idx >= n) idx -= n;
                    }
                    o += idx * static_cast<I>(sd.stride[d]);
                }
            }
        }
        const double v = src[j];
        if constexpr (std::is_same<To, DW>::value) {
            // the double-word right-hand side of the mixed solve: the
            // integer split below, hi + lo = v to about 2^-46 relative
            float h, l;
            split_double(v, h, l);
            dst[o] = DW(h, l);
        } else {
            if constexpr (sizeof(To) == 4) {
                if (dlo) {
                    // integer split (no FP64 instructions): dst + dlo = v to
                    // about 2^-46 relative
                    float h, l;
                    split_double(v, h, l);
                    dst[o] = h;
                    dst2[o] = h;
                    dlo[o] = l;
                    continue;
                }
            }
            dst[o] = static_cast<To>(v);
        }
    }
}

// The mixed solve's double-word solution as the table's two FP32 arrays:
// control point = hi + lo.
__global__ void __launch_bounds__(256) dw_unpack_kernel(const DW* __restrict__ w, float* __restrict__ hi,
                                                        float* __restrict__ lo, int64_t n) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const DW v = w[i];
        hi[i] = v.hi;
        lo[i] = v.lo;
    }
}

bool shift_identity(const ShiftDesc& sd) {
    if (sd.channels != 1) return false;
    for (int d = 0; d < sd.dim; ++d)
        if (sd.shift[d]) return false;
    return true;
}

// Position of element e along an axis of n points and stride S: (e / S) % n.
// (32-bit indices: fast division; 64-bit ones: plain division.)
struct AxisPos {
    FastDiv byS, byN;
    int64_t S64, n64;
    __device__ __forceinline__ uint32_t operator()(uint32_t e) const {
        const uint32_t q = byS.div(e);
        return q - byN.div(q) * byN.d;
    }
    __device__ __forceinline__ int64_t operator()(int64_t e) const { return (e / S64) % n64; }
};

}  // namespace

INTP_DEFINE_WARM_CAP_SETTER(set_warm_cap_solve)

int take_device_error(cudaStream_t s) {
    int v = 0, zero = 0;
    if (cudaMemcpyFromSymbolAsync(&v, g_device_error, sizeof(int), 0, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return 0;
    cudaMemcpyToSymbolAsync(g_device_error, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
    return v;
}

cudaError_t launch_line_solve_f64(double* x, int64_t n, int64_t S, int64_t nlines, int p, int q, bool cyclic,
                                  const double* lower, const double* upper, const double* dinv, const double* bottom,
                                  const double* right, cudaStream_t s, int64_t clo, int64_t chi,
                                  int64_t zside) {
    FactorView<double> f{n, lower, upper, dinv, bottom, right, clo, chi, zside};
    return launch_solve_r<double>(x, n, S, nlines, p, q, cyclic, f, s);
}

cudaError_t launch_line_solve_f32(float* x, int64_t n, int64_t S, int64_t nlines, int p, int q, bool cyclic,
                                  const float* lower, const float* upper, const float* dinv, const float* bottom,
                                  const float* right, cudaStream_t s, int64_t clo, int64_t chi,
                                  int64_t zside) {
    FactorView<float> f{n, lower, upper, dinv, bottom, right, clo, chi, zside};
    return launch_solve_r<float>(x, n, S, nlines, p, q, cyclic, f, s);
}

cudaError_t launch_line_solve_dw(DW* x, int64_t n, int64_t S, int64_t nlines, int p, int q, bool cyclic,
                                 const DW* lower, const DW* upper, const DW* dinv, const DW* bottom, const DW* right,
                                 cudaStream_t s, int64_t clo, int64_t chi, int64_t zside) {
    FactorView<DW> f{n, lower, upper, dinv, bottom, right, clo, chi, zside};
    return launch_solve_r<DW>(x, n, S, nlines, p, q, cyclic, f, s);
}

cudaError_t launch_shift_copy_f64_f64(const double* src, double* dst, const ShiftDesc& sd,
                                      cudaStream_t s) {
    const int64_t N = sd.total * sd.channels;
    const int grid = grid_for(N, 256, 152 * 16);
    const int id = shift_identity(sd) ? 1 : 0;
    if (N <= kIndex32Max)
        shift_copy_kernel<double, uint32_t><<<grid, 256, 0, s>>>(src, dst, nullptr, nullptr, sd, id);
    else
        shift_copy_kernel<double, int64_t><<<grid, 256, 0, s>>>(src, dst, nullptr, nullptr, sd, id);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_shift_copy_f64_dw(const double* src, DW* dst, const ShiftDesc& sd, cudaStream_t s) {
    const int64_t N = sd.total * sd.channels;
    const int grid = grid_for(N, 256, 152 * 16);
    const int id = shift_identity(sd) ? 1 : 0;
    if (N <= kIndex32Max)
        shift_copy_kernel<DW, uint32_t><<<grid, 256, 0, s>>>(src, dst, nullptr, nullptr, sd, id);
    else
        shift_copy_kernel<DW, int64_t><<<grid, 256, 0, s>>>(src, dst, nullptr, nullptr, sd, id);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_dw_unpack(const DW* w, float* hi, float* lo, int64_t n, cudaStream_t s) {
    dw_unpack_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(w, hi, lo, n);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_shift_copy_f64_f32(const double* src, float* dst, float* dst_lo, float* dst2, const ShiftDesc& sd,
                                      cudaStream_t s) {
    const int64_t N = sd.total * sd.channels;
    const int grid = grid_for(N, 256, 152 * 16);
    const int id = shift_identity(sd) ? 1 : 0;
    if (N <= kIndex32Max)
        shift_copy_kernel<float, uint32_t><<<grid, 256, 0, s>>>(src, dst, dst_lo, dst2, sd, id);
    else
        shift_copy_kernel<float, int64_t><<<grid, 256, 0, s>>>(src, dst, dst_lo, dst2, sd, id);
    note_launch();
    return cudaGetLastError();
}


}  // namespace intp_gb300
