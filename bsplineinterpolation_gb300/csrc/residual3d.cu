// Fused residual of the mixed form's refinement for 3D tables: r = F - (A_0 x
// A_1 x A_2) c in one kernel instead of one pass per axis.
//
// The per-axis passes (solve_kernels.cu, residual_pass_kernel) apply the
// collocation stencil of axis 2, then axis 1, then axis 0, each reading and
// writing a double-float array of the whole mesh (8 bytes per value each
// way). Here a CTA owns a column block of 16 (axis 1) x 32 (axis 2) outputs
// and a segment of axis 0, and marches along axis 0 one slice at a time:
//
//   load:    the slice's (16 + 2B) x (32 + 2B) block of c (and of its
//            remainders) into shared memory, wrapped on periodic axes;
//   x pass:  axis-2 stencil on every row of the block (16 + 2B rows);
//   y pass:  axis-1 stencil -> one slot of a ring of 2B + 1 slices;
//   z pass:  once the slices z - b_0 .. z + b_0 are in the ring, output z is
//            F - (axis-0 stencil over them), rounded to FP32.
//
// Every element's arithmetic is that of the per-axis passes -- the same
// Dot2 accumulations (refine_df.cuh) in the same tap order on the same
// operands -- so the control points are bit-identical to the pass-by-pass
// build (and to the batched build, which shares those operations); only the
// intermediates stay on chip. Taps whose coefficient is zero are skipped,
// which is also what keeps reads of slices or columns outside a
// non-periodic axis from ever happening.
#include <cuda_runtime.h>

#include <cstdint>

#include "launch.hpp"
#include "refine_df.cuh"

namespace intp_gb300 {

namespace {

constexpr int kR3Threads = 256;
constexpr int kR3TY = 16;  // axis-1 outputs per CTA
constexpr int kR3TX = 32;  // axis-2 outputs per CTA
constexpr int kR3ZS = 32;  // axis-0 outputs per CTA (a segment of the march)

__device__ __forceinline__ int wrap_mod(int i, int n) {
    const int m = i % n;
    return m < 0 ? m + n : m;
}

// Axis description: points, stencil half-width, periodicity, the stencil
// rows (2 band + 1 double-float taps per row).
struct R3Axis {
    int n;
    int band;
    int periodic;
    const float2* val;
};

// Stencil row of one output index in registers: the taps, zero taps as
// zeros (skipped by the accumulation, as the per-axis passes skip them).
template <int BMAX>
struct R3Row {
    float2 a[2 * BMAX + 1];
    __device__ __forceinline__ void load(const R3Axis& ax, int i, bool valid) {
        const int w = 2 * ax.band + 1;
#pragma unroll
        for (int d = 0; d < 2 * BMAX + 1; ++d)
            a[d] = (valid && d < w) ? __ldg(ax.val + static_cast<int64_t>(i) * w + d) : make_float2(0.0f, 0.0f);
    }
};

// Lane = axis-2 position within the block's 32 columns; warp w owns rows
// w, w + 8, ... of each pass. The axis-2 and axis-1 stencil rows of a
// thread's outputs do not change along the march and stay in registers.
template <int BMAX, bool HAS_LO>
__global__ void __launch_bounds__(kR3Threads) residual3d_kernel(const float* __restrict__ c_hi,
                                                                const float* __restrict__ c_lo,
                                                                const float* __restrict__ rhs_hi,
                                                                const float* __restrict__ rhs_lo,
                                                                float* __restrict__ r, R3Axis az, R3Axis ay,
                                                                R3Axis ax, int zsegs) {
    constexpr int W = 2 * BMAX + 1;  // ring slots (>= 2 b_0 + 1) and taps per row
    constexpr int IY = kR3TY + 2 * BMAX, IX = kR3TX + 2 * BMAX;
    constexpr int kWarps = kR3Threads / 32;
    constexpr int kYRows = kR3TY / kWarps;  // y-pass rows per warp
    static_assert(kR3TX == 32 && kR3TY % kWarps == 0, "lane = column, warps share the rows");
    __shared__ float2 inp[IY][IX];
    __shared__ float2 s1[IY][kR3TX];
    __shared__ float2 ring[W][kR3TY][kR3TX];
    const int nx = ax.n, ny = ay.n, nz = az.n;
    const int ch = blockIdx.z / zsegs, zseg = blockIdx.z - ch * zsegs;
    const int64_t sz = static_cast<int64_t>(nx) * ny;
    const int64_t cbase = static_cast<int64_t>(ch) * nz * sz;  // channel block (channel-major storage)
    const int x0 = blockIdx.x * kR3TX, y0 = blockIdx.y * kR3TY, z0 = zseg * kR3ZS;
    const int z1 = z0 + kR3ZS < nz ? z0 + kR3ZS : nz;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int gx = x0 + lane;
    const bool xin = gx < nx;
    R3Row<BMAX> rx;
    rx.load(ax, gx, xin);
    R3Row<BMAX> ry[kYRows];
#pragma unroll
    for (int k = 0; k < kYRows; ++k) ry[k].load(ay, y0 + warp + k * kWarps, y0 + warp + k * kWarps < ny);
    const int xo = BMAX - ax.band, yo = BMAX - ay.band;  // tap d reads halo column / row (out + offset + d)
    for (int zz = z0 - az.band; zz < z1 + az.band; ++zz) {
        // the slice: wrapped on a periodic axis; outside a non-periodic one it
        // is never read (its taps are zero) and is not computed
        int zg = zz;
        bool zvalid = true;
        if (az.periodic)
            zg = wrap_mod(zz, nz);
        else
            zvalid = zz >= 0 && zz < nz;
        if (zvalid) {
            const int64_t zoff = cbase + static_cast<int64_t>(zg) * sz;
            for (int e = tid; e < IY * IX; e += kR3Threads) {
                const int iy = e / IX, ix = e - iy * IX;
                int gy = y0 - BMAX + iy, gxx = x0 - BMAX + ix;
                bool ok = true;
                if (ay.periodic)
                    gy = wrap_mod(gy, ny);
                else
                    ok = ok && gy >= 0 && gy < ny;
                if (ax.periodic)
                    gxx = wrap_mod(gxx, nx);
                else
                    ok = ok && gxx >= 0 && gxx < nx;
                float2 v = make_float2(0.0f, 0.0f);
                if (ok) {
                    const int64_t j = zoff + static_cast<int64_t>(gy) * nx + gxx;
                    v.x = __ldg(c_hi + j);
                    if (HAS_LO) v.y = __ldg(c_lo + j);
                }
                inp[iy][ix] = v;
            }
            __syncthreads();
            // axis 2 on every row of the block
            for (int iy = warp; iy < IY; iy += kWarps) {
                Dot2 acc{0.0f, 0.0f};
#pragma unroll
                for (int d = 0; d < W; ++d) {
                    if (rx.a[d].x != 0.0f) {
                        const float2 v = inp[iy][lane + xo + d];
                        dot2_add<HAS_LO>(acc, rx.a[d], v.x, v.y);
                    }
                }
                const DF dv = dot2_value(acc);
                s1[iy][lane] = make_float2(dv.hi, dv.lo);
            }
            __syncthreads();
            // axis 1 -> the slice's ring slot
            float2(*slot)[kR3TX] = ring[wrap_mod(zz, W)];
#pragma unroll
            for (int k = 0; k < kYRows; ++k) {
                const int y = warp + k * kWarps;
                Dot2 acc{0.0f, 0.0f};
#pragma unroll
                for (int d = 0; d < W; ++d) {
                    if (ry[k].a[d].x != 0.0f) {
                        const float2 v = s1[y + yo + d][lane];
                        dot2_add<true>(acc, ry[k].a[d], v.x, v.y);
                    }
                }
                const DF dv = dot2_value(acc);
                slot[y][lane] = make_float2(dv.hi, dv.lo);
            }
        }
        __syncthreads();
        // axis 0 for the output whose last slice this was
        const int z = zz - az.band;
        if (z >= z0 && z < z1) {
            R3Row<BMAX> rz;
            rz.load(az, z, true);
            const int zo = z - az.band;  // slice of tap 0
#pragma unroll
            for (int k = 0; k < kYRows; ++k) {
                const int y = warp + k * kWarps, gy = y0 + y;
                if (gy < ny && xin) {
                    const int64_t j = cbase + static_cast<int64_t>(z) * sz + static_cast<int64_t>(gy) * nx + gx;
                    Dot2 acc{__ldg(rhs_hi + j), __ldg(rhs_lo + j)};
#pragma unroll
                    for (int d = 0; d < W; ++d) {
                        if (rz.a[d].x != 0.0f) {
                            const float2 a = make_float2(-rz.a[d].x, -rz.a[d].y);
                            const float2 v = ring[wrap_mod(zo + d, W)][y][lane];
                            dot2_add<true>(acc, a, v.x, v.y);
                        }
                    }
                    r[j] = __fadd_rn(acc.s, acc.c);
                }
            }
        }
        // the next slice overwrites a ring slot only after its load and its
        // x pass (two barriers away)
    }
}

template <int BMAX>
cudaError_t launch_b(const float* c_hi, const float* c_lo, const float* rhs_hi, const float* rhs_lo, float* r,
                     const R3Axis& az, const R3Axis& ay, const R3Axis& ax, int channels, cudaStream_t s) {
    const int zsegs = (az.n + kR3ZS - 1) / kR3ZS;
    const dim3 grid((ax.n + kR3TX - 1) / kR3TX, (ay.n + kR3TY - 1) / kR3TY, zsegs * channels);
    if (c_lo)
        residual3d_kernel<BMAX, true><<<grid, kR3Threads, 0, s>>>(c_hi, c_lo, rhs_hi, rhs_lo, r, az, ay, ax, zsegs);
    else
        residual3d_kernel<BMAX, false><<<grid, kR3Threads, 0, s>>>(c_hi, c_lo, rhs_hi, rhs_lo, r, az, ay, ax, zsegs);
    note_launch();
    return cudaGetLastError();
}

}  // namespace

bool residual3d_supported(const int* n, const int* band, int channels) {
    int bmax = 0;
    for (int d = 0; d < 3; ++d) {
        if (n[d] < 1 || band[d] < 0) return false;
        if (band[d] > bmax) bmax = band[d];
    }
    // grid limits: axis-1 blocks and axis-0 segments x channels
    if ((n[1] + kR3TY - 1) / kR3TY > 65535) return false;
    if (static_cast<int64_t>((n[0] + kR3ZS - 1) / kR3ZS) * channels > 65535) return false;
    // static shared memory of the widest instantiation (BMAX = 3) stays below 48 KB
    return bmax <= 3;
}

cudaError_t launch_residual3d(const float* c_hi, const float* c_lo, const float* rhs_hi, const float* rhs_lo, float* r,
                              const int* n, const int* band, const int* periodic, const float2* const* val,
                              int channels, cudaStream_t s) {
    if (!residual3d_supported(n, band, channels)) return cudaErrorInvalidValue;
    const R3Axis az{n[0], band[0], periodic[0], val[0]};
    const R3Axis ay{n[1], band[1], periodic[1], val[1]};
    const R3Axis ax{n[2], band[2], periodic[2], val[2]};
    int bmax = 0;
    for (int d = 0; d < 3; ++d) bmax = band[d] > bmax ? band[d] : bmax;
    if (bmax <= 2) return launch_b<2>(c_hi, c_lo, rhs_hi, rhs_lo, r, az, ay, ax, channels, s);
    return launch_b<3>(c_hi, c_lo, rhs_hi, rhs_lo, r, az, ay, ax, channels, s);
}

}  // namespace intp_gb300
