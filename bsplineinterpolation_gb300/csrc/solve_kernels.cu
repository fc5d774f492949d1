// Control-point solve: per-axis band / cyclic-band substitution over every
// mesh line (InterpolationTemplate.hpp:448-580, BandLU.hpp:120-143 and
// :215-259), plus the double-float residual of mixed-precision refinement.
//
// A mesh of shape N_0 x ... x N_{D-1} is processed one axis at a time. Along
// axis a the lines are indexed by (outer o, inner t): element k of a line is
// at o*N_a*S + k*S + t with S = prod_{d>a} N_d. One thread owns one line;
// adjacent threads own adjacent t, so for S >= 32 every step of the
// substitution is a coalesced warp-wide access. The contiguous axis (S = 1)
// is staged through shared memory so it is read and written coalesced too.
// The reference instead rotates the whole tensor after each axis pass
// (:537-543); solving in place along strided lines needs no rotation. The
// substitution itself is solve_line (solve_line.cuh).
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

template <class R, int P, int Q, bool CYC>
__global__ void __launch_bounds__(128) solve_strided_kernel(R* __restrict__ x, int64_t n, int64_t S,
                                                            int64_t nlines, FactorView<R> f) {
    for (int64_t l = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; l < nlines;
         l += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t o = l / S, t = l - o * S;
        StridedLine<R> line{x + o * n * S + t, S};
        solve_line<R, P, Q, CYC>(f, line);
    }
}

// Contiguous lines (S = 1): a block stages 32 lines x n into shared memory
// (row pitch n+1, conflict-free per-lane access), solves, writes back.
template <class R, int P, int Q, bool CYC>
__global__ void __launch_bounds__(32) solve_contig_kernel(R* __restrict__ x, int64_t n, int64_t nlines,
                                                          FactorView<R> f) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    R* tile = reinterpret_cast<R*>(smem_raw);
    const int64_t pitch = n + 1;
    const int lane = threadIdx.x;
    for (int64_t l0 = blockIdx.x * 32LL; l0 < nlines; l0 += gridDim.x * 32LL) {
        const int rows = static_cast<int>(nlines - l0 < 32 ? nlines - l0 : 32);
        const R* src = x + l0 * n;
        for (int r = 0; r < rows; ++r)
            for (int64_t k = lane; k < n; k += 32) tile[r * pitch + k] = src[r * n + k];
        __syncwarp();
        if (lane < rows) solve_line<R, P, Q, CYC>(f, SmemLine<R>{tile + lane * pitch});
        __syncwarp();
        R* dst = x + l0 * n;
        for (int r = 0; r < rows; ++r)
            for (int64_t k = lane; k < n; k += 32) dst[r * n + k] = tile[r * pitch + k];
        __syncwarp();
    }
}

template <class R, int P, int Q, bool CYC>
cudaError_t launch_solve_pq_fallback(R* x, int64_t n, int64_t S, int64_t nlines, const FactorView<R>& f,
                                     cudaStream_t s);

// ---- tiled solves: one warp stages 32 lines in shared memory ----

// Column of a [n][32] tile: element k of lane l at base[k*32 + l].
template <class R>
struct TileColumn {
    R* base;
    __device__ __forceinline__ R load(int64_t k) const { return base[k * 32]; }
    __device__ __forceinline__ void store(int64_t k, R v) const { base[k * 32] = v; }
};

// Strided axis (S % (16/sizeof(R)) == 0): the tile holds 32 adjacent lines
// (t0 .. t0+31 for one outer index o); row k of the tile is the 32 contiguous
// elements k*S + t0 .. + 31, moved by one TMA bulk copy each way.
template <class R, int P, int Q, bool CYC>
__global__ void __launch_bounds__(32) solve_tile_strided_kernel(R* __restrict__ x, int64_t n, int64_t S,
                                                                int64_t tiles_per_o, int64_t ntiles,
                                                                FactorView<R> f) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    R* tile = reinterpret_cast<R*>(smem_raw);
    const int lane = threadIdx.x;
    if (lane == 0) mbar_init(&bar, 1);
    __syncwarp();
    uint32_t phase = 0;
    for (int64_t tl = blockIdx.x; tl < ntiles; tl += gridDim.x) {
        const int64_t o = tl / tiles_per_o, t0 = (tl - o * tiles_per_o) * 32;
        const int w = static_cast<int>(S - t0 < 32 ? S - t0 : 32);
        const uint32_t row_bytes = static_cast<uint32_t>(w * sizeof(R));
        R* base = x + o * n * S + t0;
        if (lane == 0) mbar_expect_tx(&bar, row_bytes * static_cast<uint32_t>(n));
        __syncwarp();
        for (int64_t k = lane; k < n; k += 32) bulk_load(tile + k * 32, base + k * S, row_bytes, &bar);
        if (!mbar_wait(&bar, phase)) {
            mbar_wait(&bar, phase);  // give the copies in flight a second bounded wait
            return;
        }
        phase ^= 1u;
        if (lane < w) solve_line<R, P, Q, CYC>(f, TileColumn<R>{tile + lane});
        __syncwarp();
        fence_async_smem();
        __syncwarp();
        for (int64_t k = lane; k < n; k += 32) bulk_store(base + k * S, tile + k * 32, row_bytes);
        bulk_store_commit();
        bulk_store_wait_read();
        __syncwarp();
    }
    bulk_store_wait_all();
}

// Contiguous axis (S = 1): 32 lines of n elements copied element-wise with
// cp.async into rows of pitch n+1, so lane l reading element k of line l
// touches bank (l + k) mod 32: no conflicts.
template <class R, int P, int Q, bool CYC>
__global__ void __launch_bounds__(32) solve_tile_contig_kernel(R* __restrict__ x, int64_t n, int64_t nlines,
                                                               FactorView<R> f) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    R* tile = reinterpret_cast<R*>(smem_raw);
    const int64_t pitch = n + 1;
    const int lane = threadIdx.x;
    for (int64_t l0 = blockIdx.x * 32LL; l0 < nlines; l0 += gridDim.x * 32LL) {
        const int rows = static_cast<int>(nlines - l0 < 32 ? nlines - l0 : 32);
        const R* src = x + l0 * n;
        for (int r = 0; r < rows; ++r)
            for (int64_t k = lane; k < n; k += 32) cp_async<sizeof(R)>(tile + r * pitch + k, src + r * n + k);
        cp_async_wait_all();
        __syncwarp();
        if (lane < rows) solve_line<R, P, Q, CYC>(f, SmemLine<R>{tile + lane * pitch});
        __syncwarp();
        R* dst = x + l0 * n;
        for (int r = 0; r < rows; ++r)
            for (int64_t k = lane; k < n; k += 32) dst[r * n + k] = tile[r * pitch + k];
        __syncwarp();
    }
}

int sm_count_solve() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    }
    return n;
}

constexpr size_t kTileSmemLimit = 200 * 1024;

template <class R, int P, int Q, bool CYC>
cudaError_t launch_solve_pq(R* x, int64_t n, int64_t S, int64_t nlines, const FactorView<R>& f,
                            cudaStream_t s) {
    const size_t tile_bytes = static_cast<size_t>(n) * 32 * sizeof(R);
    const bool aligned = (S * static_cast<int64_t>(sizeof(R))) % 16 == 0 &&
                         (reinterpret_cast<uintptr_t>(x) % 16) == 0;
    if (S >= 32 && aligned && tile_bytes <= kTileSmemLimit) {
        auto k = solve_tile_strided_kernel<R, P, Q, CYC>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(tile_bytes));
        if (e != cudaSuccess) return e;
        const int64_t tiles_per_o = (S + 31) / 32;
        const int64_t ntiles = (nlines / S) * tiles_per_o;
        const int per_sm = static_cast<int>(std::max<size_t>(1, 220 * 1024 / (tile_bytes + 1024)));
        const int grid = static_cast<int>(std::min<int64_t>(ntiles, int64_t{sm_count_solve()} * per_sm));
        k<<<grid, 32, tile_bytes, s>>>(x, n, S, tiles_per_o, ntiles, f);
        note_launch();
        return cudaGetLastError();
    }
    const size_t ctile = static_cast<size_t>(32) * static_cast<size_t>(n + 1) * sizeof(R);
    if (S == 1 && ctile <= kTileSmemLimit) {
        auto k = solve_tile_contig_kernel<R, P, Q, CYC>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(ctile));
        if (e != cudaSuccess) return e;
        const int per_sm = static_cast<int>(std::max<size_t>(1, 220 * 1024 / (ctile + 1024)));
        const int64_t ntiles = (nlines + 31) / 32;
        const int grid = static_cast<int>(std::min<int64_t>(ntiles, int64_t{sm_count_solve()} * per_sm));
        k<<<grid, 32, ctile, s>>>(x, n, nlines, f);
        note_launch();
        return cudaGetLastError();
    }
    return launch_solve_pq_fallback<R, P, Q, CYC>(x, n, S, nlines, f, s);
}

template <class R, int P, int Q, bool CYC>
cudaError_t launch_solve_pq_fallback(R* x, int64_t n, int64_t S, int64_t nlines, const FactorView<R>& f,
                                     cudaStream_t s) {
    const size_t smem = static_cast<size_t>(32) * static_cast<size_t>(n + 1) * sizeof(R);
    if (S == 1 && smem <= 96 * 1024) {
        auto k = solve_contig_kernel<R, P, Q, CYC>;
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 static_cast<int>(smem));
            if (e != cudaSuccess) return e;
        }
        const int grid = grid_for(nlines, 32, 152 * 64);
        k<<<grid, 32, smem, s>>>(x, n, nlines, f);
        note_launch();
        return cudaGetLastError();
    }
    const int grid = grid_for(nlines, 128, 152 * 64);
    solve_strided_kernel<R, P, Q, CYC><<<grid, 128, 0, s>>>(x, n, S, nlines, f);
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
// accumulation: out = A_axis in as a double-float, or on the last pass
// (FINAL) r = rhs - A_axis in rounded to FP32 -- the correction solve's
// right-hand side. HAS_LO: the input is double-float (else plain FP32). One
// thread per output element; adjacent threads read adjacent elements of
// every tap.
template <class I, bool HAS_LO, bool FINAL>
__global__ void __launch_bounds__(256) residual_pass_kernel(const float* __restrict__ in_hi,
                                                            const float* __restrict__ in_lo, float* __restrict__ out_hi,
                                                            float* __restrict__ out_lo,
                                                            const float* __restrict__ rhs_hi,
                                                            const float* __restrict__ rhs_lo, float* __restrict__ r,
                                                            AxisPos pos, I S, I N, int width,
                                                            const int32_t* __restrict__ col,
                                                            const float2* __restrict__ val) {
    for (I e = blockIdx.x * static_cast<I>(blockDim.x) + threadIdx.x; e < N;
         e += static_cast<I>(gridDim.x) * blockDim.x) {
        const I i = pos(e);
        Dot2 acc{0.0f, 0.0f};
        if (FINAL) acc = Dot2{rhs_hi[e], rhs_lo[e]};
        dot2_row<HAS_LO, I>(acc, FINAL ? -1.0f : 1.0f, in_hi, in_lo, e - i * S, static_cast<int>(i), S, width, col,
                            val);
        if (FINAL) {
            r[e] = __fadd_rn(acc.s, acc.c);
        } else {
            const DF v = dot2_value(acc);
            out_hi[e] = v.hi;
            out_lo[e] = v.lo;
        }
    }
}

template <class I, bool HAS_LO, bool FINAL>
void launch_residual_t(const float* in_hi, const float* in_lo, float* out_hi, float* out_lo, const float* rhs_hi,
                       const float* rhs_lo, float* r, int64_t n, int64_t S, int64_t N, int width, const int32_t* col,
                       const float2* val, cudaStream_t s) {
    AxisPos pos{};
    if (N <= kIndex32Max) {
        pos.byS = FastDiv::make(static_cast<uint32_t>(S));
        pos.byN = FastDiv::make(static_cast<uint32_t>(n));
    }
    pos.S64 = S;
    pos.n64 = n;
    residual_pass_kernel<I, HAS_LO, FINAL><<<grid_for(N, 256, 152 * 16), 256, 0, s>>>(
        in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, pos, static_cast<I>(S), static_cast<I>(N), width, col, val);
}

template <class I>
void launch_residual_i(const float* in_hi, const float* in_lo, float* out_hi, float* out_lo, const float* rhs_hi,
                       const float* rhs_lo, float* r, int64_t n, int64_t S, int64_t N, int width, const int32_t* col,
                       const float2* val, cudaStream_t s) {
    const bool lo = in_lo != nullptr, fin = rhs_hi != nullptr;
    if (lo && fin)
        launch_residual_t<I, true, true>(in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, n, S, N, width, col, val, s);
    else if (lo)
        launch_residual_t<I, true, false>(in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, n, S, N, width, col, val, s);
    else if (fin)
        launch_residual_t<I, false, true>(in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, n, S, N, width, col, val, s);
    else
        launch_residual_t<I, false, false>(in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, n, S, N, width, col, val,
                                           s);
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

int take_device_error(cudaStream_t s) {
    int v = 0, zero = 0;
    if (cudaMemcpyFromSymbolAsync(&v, g_device_error, sizeof(int), 0, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return 0;
    cudaMemcpyToSymbolAsync(g_device_error, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
    return v;
}

cudaError_t launch_line_solve_f64(double* x, int64_t n, int64_t S, int64_t nlines, int p, int q,
                                  bool cyclic, const double* lower, const double* upper,
                                  const double* dinv, const double* bottom, const double* right,
                                  cudaStream_t s) {
    FactorView<double> f{n, lower, upper, dinv, bottom, right};
    return launch_solve_r<double>(x, n, S, nlines, p, q, cyclic, f, s);
}

cudaError_t launch_line_solve_f32(float* x, int64_t n, int64_t S, int64_t nlines, int p, int q,
                                  bool cyclic, const float* lower, const float* upper,
                                  const float* dinv, const float* bottom, const float* right,
                                  cudaStream_t s) {
    FactorView<float> f{n, lower, upper, dinv, bottom, right};
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
                                 int width, const int32_t* col, const float2* val, cudaStream_t s) {
    if (N <= kIndex32Max)
        launch_residual_i<uint32_t>(in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, n, S, N, width, col, val, s);
    else
        launch_residual_i<int64_t>(in_hi, in_lo, out_hi, out_lo, rhs_hi, rhs_lo, r, n, S, N, width, col, val, s);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_correct(float* c, float* lo, const float* corr, int64_t n, bool has_lo, cudaStream_t s) {
    correct_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(c, lo, corr, n, has_lo ? 1 : 0);
    note_launch();
    return cudaGetLastError();
}

}  // namespace intp_gb300
