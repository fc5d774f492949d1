// Control-point solve: per-axis band / cyclic-band substitution over every
// mesh line (InterpolationTemplate.hpp:448-580, BandLU.hpp:120-143 and
// :215-259), plus the double-float residual of mixed-precision refinement.
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
#include "refine_df.cuh"
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
__global__ void __launch_bounds__(kSolveWarps * 32) solve_warp_strided_kernel(R* __restrict__ x, int64_t n,
                                                                              int64_t S, int64_t nlines,
                                                                              FactorView<R> f) {
    for (int64_t l = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; l < nlines;
         l += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t o = l / S, t = l - o * S;
        solve_line_chunked<R, P, Q, CYC, line_chunk<R>()>(f, StridedChunks<R>{x + o * n * S + t, S});
    }
}

// Contiguous axis (S = 1): one warp per 32 consecutive lines.
template <class R, int P, int Q, bool CYC>
__global__ void __launch_bounds__(kSolveWarps * 32, 4) solve_warp_contig_kernel(R* __restrict__ x, int64_t n,
                                                                             int64_t nlines, FactorView<R> f) {
    __shared__ R stage[kSolveWarps][32 * 33];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t ngroups = (nlines + 31) / 32;
    for (int64_t g = blockIdx.x * static_cast<int64_t>(kSolveWarps) + warp; g < ngroups;
         g += static_cast<int64_t>(gridDim.x) * kSolveWarps) {
        const int64_t l0 = g * 32;
        const int rows = static_cast<int>(nlines - l0 < 32 ? nlines - l0 : 32);
        WarpContigChunks<R> io{x + l0 * n, n, rows, stage[warp], lane};
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

// One residual pass of the mixed form's refinement along an axis of n points
// and stride S, over all N values (channel blocks included), with Dot2
// accumulation over the axis' band stencil (dot2_band_row, the operations of
// the batched residual): out = A_axis in as a double-float, or on the last
// pass (FINAL) r = rhs - A_axis in rounded to FP32 -- the correction solve's
// right-hand side. HAS_LO: the input is double-float (else plain FP32). One
// thread per output element, kResidualIlp elements per loop trip (independent loads
// in flight); the columns are computed, not loaded, and on a strided axis
// the warp's coefficient loads are broadcasts.
constexpr int kResidualIlp = 4;

// One element pair of a residual pass: elements e0, e1 (e1 >= N: a dummy
// lane with zero coefficients and operands, never stored) as the two lanes
// of the packed accumulator. Each lane applies dot2_band_row_t's taps in its
// order; a tap that is zero in one lane only adds an exact zero there (the
// running sum and error term keep their values), so each lane's result is
// that of the scalar pass.
template <class I, int BAND, bool PERIODIC, bool HAS_LO, bool FINAL>
__device__ __forceinline__ void residual_pair(const float* __restrict__ in_hi, const float* __restrict__ in_lo,
                                              float* __restrict__ out_hi, float* __restrict__ out_lo,
                                              const float* __restrict__ rhs_hi, const float* __restrict__ rhs_lo,
                                              float* __restrict__ r, const AxisPos& pos, I S, I N, int n,
                                              const float2* __restrict__ val, I e0, I e1) {
    constexpr int W = 2 * BAND + 1;
    const bool v1 = e1 < N;
    const I i0 = pos(e0), i1 = v1 ? pos(e1) : I(0);
    const I b0 = e0 - i0 * S, b1 = v1 ? e1 - i1 * S : I(0);
    Dot2x2 acc{make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f)};
    if (FINAL) {
        acc.s = make_float2(rhs_hi[e0], v1 ? rhs_hi[e1] : 0.0f);
        acc.c = make_float2(rhs_lo[e0], v1 ? rhs_lo[e1] : 0.0f);
    }
    const float2* __restrict__ row0 = val + static_cast<int64_t>(i0) * W;
    const float2* __restrict__ row1 = val + static_cast<int64_t>(i1) * W;
#pragma unroll
    for (int d = 0; d < W; ++d) {
        float2 a0 = __ldg(row0 + d);
        float2 a1 = v1 ? __ldg(row1 + d) : make_float2(0.0f, 0.0f);
        const bool z0 = a0.x == 0.0f, z1 = a1.x == 0.0f;
        if (z0 && z1) continue;
        if (FINAL) {
            a0.x = -a0.x;
            a0.y = -a0.y;
            a1.x = -a1.x;
            a1.y = -a1.y;
        }
        float2 xh = make_float2(0.0f, 0.0f), xl = make_float2(0.0f, 0.0f);
        if (!z0) {
            int c = static_cast<int>(i0) - BAND + d;
            if (PERIODIC) c = c < 0 ? c + n : (c >= n ? c - n : c);
            const I j = b0 + static_cast<I>(c) * S;
            xh.x = __ldg(in_hi + j);
            if (HAS_LO) xl.x = __ldg(in_lo + j);
        }
        if (!z1) {
            int c = static_cast<int>(i1) - BAND + d;
            if (PERIODIC) c = c < 0 ? c + n : (c >= n ? c - n : c);
            const I j = b1 + static_cast<I>(c) * S;
            xh.y = __ldg(in_hi + j);
            if (HAS_LO) xl.y = __ldg(in_lo + j);
        }
        dot2_add2<HAS_LO>(acc, make_float2(a0.x, a1.x), make_float2(a0.y, a1.y), xh, xl);
    }
    if (FINAL) {
        const float2 v = __fadd2_rn(acc.s, acc.c);
        r[e0] = v.x;
        if (v1) r[e1] = v.y;
    } else {
        float2 h, l;
        df_two_sum2(acc.s, acc.c, h, l);
        out_hi[e0] = h.x;
        out_lo[e0] = l.x;
        if (v1) {
            out_hi[e1] = h.y;
            out_lo[e1] = l.y;
        }
    }
}

template <class I, int BAND, bool PERIODIC, bool HAS_LO, bool FINAL>
__global__ void __launch_bounds__(256) residual_pass_kernel(const float* __restrict__ in_hi,
                                                            const float* __restrict__ in_lo, float* __restrict__ out_hi,
                                                            float* __restrict__ out_lo,
                                                            const float* __restrict__ rhs_hi,
                                                            const float* __restrict__ rhs_lo, float* __restrict__ r,
                                                            AxisPos pos, I S, I N, int n,
                                                            const float2* __restrict__ val) {
    const I stride = static_cast<I>(gridDim.x) * blockDim.x;
    for (I e0 = blockIdx.x * static_cast<I>(blockDim.x) + threadIdx.x; e0 < N; e0 += kResidualIlp * stride) {
#pragma unroll
        for (int u = 0; u < kResidualIlp; u += 2) {
            const I e = e0 + u * stride;
            if (e < N)
                residual_pair<I, BAND, PERIODIC, HAS_LO, FINAL>(in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, pos, S,
                                                                N, n, val, e, e + stride);
        }
    }
}

template <int BAND, bool PERIODIC, bool HAS_LO, bool FINAL>
void launch_residual_t(const float* in_hi, const float* in_lo, float* out_hi, float* out_lo, const float* rhs_hi,
                       const float* rhs_lo, float* r, int64_t n, int64_t S, int64_t N, const float2* val,
                       cudaStream_t s) {
    AxisPos pos{};
    pos.S64 = S;
    pos.n64 = n;
    const int grid = grid_for((N + kResidualIlp - 1) / kResidualIlp, 256, 152 * 16);
    if (N <= kIndex32Max) {
        pos.byS = FastDiv::make(static_cast<uint32_t>(S));
        pos.byN = FastDiv::make(static_cast<uint32_t>(n));
        residual_pass_kernel<uint32_t, BAND, PERIODIC, HAS_LO, FINAL><<<grid, 256, 0, s>>>(
            in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, pos, static_cast<uint32_t>(S), static_cast<uint32_t>(N),
            static_cast<int>(n), val);
    } else {
        residual_pass_kernel<int64_t, BAND, PERIODIC, HAS_LO, FINAL><<<grid, 256, 0, s>>>(
            in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, pos, S, N, static_cast<int>(n), val);
    }
}

template <int BAND, bool PERIODIC>
void launch_residual_bp(const float* in_hi, const float* in_lo, float* out_hi, float* out_lo, const float* rhs_hi,
                        const float* rhs_lo, float* r, int64_t n, int64_t S, int64_t N, const float2* val,
                        cudaStream_t s) {
    const bool lo = in_lo != nullptr, fin = rhs_hi != nullptr;
    if (lo && fin)
        launch_residual_t<BAND, PERIODIC, true, true>(in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, n, S, N, val, s);
    else if (lo)
        launch_residual_t<BAND, PERIODIC, true, false>(in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, n, S, N, val,
                                                       s);
    else if (fin)
        launch_residual_t<BAND, PERIODIC, false, true>(in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, n, S, N, val,
                                                       s);
    else
        launch_residual_t<BAND, PERIODIC, false, false>(in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, n, S, N, val,
                                                        s);
}

template <int BAND>
void launch_residual_b(const float* in_hi, const float* in_lo, float* out_hi, float* out_lo, const float* rhs_hi,
                       const float* rhs_lo, float* r, int64_t n, int64_t S, int64_t N, bool periodic,
                       const float2* val, cudaStream_t s) {
    if (periodic)
        launch_residual_bp<BAND, true>(in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, n, S, N, val, s);
    else
        launch_residual_bp<BAND, false>(in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, n, S, N, val, s);
}

// (c, lo) += corr, element-wise in double-float (lo taken as 0 when has_lo
// is 0: the first refinement step).
__global__ void __launch_bounds__(256) correct_kernel(float* __restrict__ c, float* __restrict__ lo,
                                                      const float* __restrict__ corr, int64_t n, int has_lo) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float h = c[i], l = has_lo ? lo[i] : 0.0f;
        df_correct(h, l, corr[i], has_lo != 0);
        c[i] = h;
        lo[i] = l;
    }
}

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

cudaError_t launch_residual_pass(const float* in_hi, const float* in_lo, float* out_hi, float* out_lo,
                                 const float* rhs_hi, const float* rhs_lo, float* r, int64_t n, int64_t S, int64_t N,
                                 int band, bool periodic, const float2* val, cudaStream_t s) {
#define INTP_RESIDUAL_CASE(B) \
    case B: launch_residual_b<B>(in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, n, S, N, periodic, val, s); break;
    switch (band) {
        INTP_RESIDUAL_CASE(0)
        INTP_RESIDUAL_CASE(1)
        INTP_RESIDUAL_CASE(2)
        INTP_RESIDUAL_CASE(3)
        INTP_RESIDUAL_CASE(4)
        INTP_RESIDUAL_CASE(5)
        INTP_RESIDUAL_CASE(6)
        default: return cudaErrorInvalidValue;
    }
#undef INTP_RESIDUAL_CASE
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_correct(float* c, float* lo, const float* corr, int64_t n, bool has_lo, cudaStream_t s) {
    correct_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(c, lo, corr, n, has_lo ? 1 : 0);
    note_launch();
    return cudaGetLastError();
}

}  // namespace intp_gb300
