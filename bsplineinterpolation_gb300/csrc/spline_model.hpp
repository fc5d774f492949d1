// Host-side model of one interpolation table: per-axis knot vectors, the
// collocation matrix of each axis and its band LU factor. These are small
// (O(n) per axis) and are built once per table on the host; everything that
// scales with the mesh (the line solves over all N^D values, evaluation) runs
// on the GPU.
//
// Semantics follow the reference library built with
// INTP_PERIODIC_NO_DUMMY_POINT (its test configuration): a periodic axis of n
// samples carries n control points and one period spans the axis range.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace intp_gb300 {

constexpr int kMaxDim = 4;
constexpr int kMaxOrder = 7;

// Band storage of an n x n matrix with lower/upper bandwidths p, q, plus the
// corner blocks of a cyclic band matrix. Entry A(i,j) of the main band lives
// at band[j*(1+p+q) + (i+q-j)] (one stored diagonal per column of `band`,
// BandMatrix.hpp:19-60). Cyclic matrices add a right block R(i, j+p-n) for
// j > i+q, (n-q-1) x p, and a bottom block S(j, i+q-n) for i > j+p,
// (n-p-1) x q (ExtendedBandMatrix, BandMatrix.hpp:99-181).
struct BandStore {
    int64_t n = 0;
    int64_t p = 0, q = 0;
    bool cyclic = false;
    std::vector<double> band, right, bottom;

    void reset(int64_t n_, int64_t p_, int64_t q_, bool cyclic_);
    double& at_main(int64_t i, int64_t j) { return band[j * (1 + p + q) + (i + q - j)]; }
    double at_main(int64_t i, int64_t j) const { return band[j * (1 + p + q) + (i + q - j)]; }
    double& at_side(int64_t i, int64_t j) {
        return j > i + q ? right[i * p + (j + p - n)] : bottom[j * q + (i + q - n)];
    }
    double at_side(int64_t i, int64_t j) const {
        return j > i + q ? right[i * p + (j + p - n)] : bottom[j * q + (i + q - n)];
    }
    double& at(int64_t i, int64_t j) {
        if (cyclic && (j > i + q || i > j + p)) return at_side(i, j);
        return at_main(i, j);
    }
    // In-place LU without pivoting in the reference's elimination order
    // (BandLU.hpp:103-118 and :159-213).
    void factorize();
    // y = A x in FP64 (BandMatrix.hpp:67-77, :148-172); used by tests.
    void multiply(const double* x, double* y) const;
};

// Per-row coefficient arrays of a factored band matrix, laid out for the GPU
// line solves. For row i:
//   lower[i*p + k] = L(i, i-p+k)        (0 outside the matrix)
//   upper[i*q + k] = U(i, i+1+k)        (0 outside the matrix)
//   dinv[i]        = 1 / U(i, i)
// Cyclic matrices add the corner blocks as dense strips:
//   bottom[r*n + j] = S(n-q+r, j) for the rows that collect the wrap-around
//                     terms during forward substitution (0 where not present)
//   right[r*n + i]  = R(i, n-p+r) for the columns that feed every earlier row
//                     during back substitution (0 where not present)
struct LineFactor {
    int64_t n = 0;
    int p = 0, q = 0;
    bool cyclic = false;
    std::vector<double> lower, upper, dinv, bottom, right;
    // rows const_lo .. const_hi-1 are bit-identical to row const_lo (the LU
    // rows of a uniform axis converge to one row away from its ends, and a
    // cyclic factor's side-band entries decay to 0 there); const_lo32 ..
    // const_hi32 the same for the FP32 roundings of the rows; empty ranges
    // where no two consecutive rows agree
    int64_t const_lo = 0, const_hi = 0;
    int64_t const_lo32 = 0, const_hi32 = 0;
    // cyclic: bottom[r*n + i] is 0 for every r and every i in zside ..
    // n-p-2 (zside32: the same for the FP32 roundings)
    int64_t zside = 0, zside32 = 0;
};

// FP32 copy of a factor entry: the rounding to nearest, with a zero result
// always +0 (the cyclic side-band entries alternate in sign as they decay,
// so their FP32 underflows would otherwise alternate between -0 and +0 and
// no two rows would agree bitwise).
inline float factor_f32(double v) {
    const float x = static_cast<float>(v);
    return x == 0.0f ? 0.0f : x;
}

// Row layout of a factored band matrix (above) for the GPU line solves.
LineFactor line_factor_from(const BandStore& lu);

// The collocation matrix itself as a row stencil (used for the residuals of
// mixed-precision refinement): row i has nonzeros A(i, col[i*w+k]) =
// val[i*w+k] for k < w, w = 1+p+q (+p+q in the cyclic case; unused slots
// have val 0 and col i).
struct RowStencil {
    int64_t n = 0;
    int width = 0;
    std::vector<int64_t> col;
    std::vector<double> val;
};

struct AxisModel {
    int64_t n = 0;        // control points (= samples, NO_DUMMY semantics)
    bool periodic = false;
    bool uniform = true;
    std::vector<double> knots;
    double range_lo = 0, range_hi = 0;  // BSpline::range_
    double dx = 0;                      // uniform axes only
    std::vector<double> input_coords;   // non-uniform axes only
    BandStore colloc;                   // collocation matrix
    BandStore lu;                       // its factor
    LineFactor factor;                  // factor in GPU row layout
    RowStencil stencil;                 // collocation rows for residuals
    double cond_est = 1.0;              // estimate of ||A||_inf ||A^-1||_inf
};

struct TableSpec {
    int dim = 0;
    int order = 0;
    bool periodic[kMaxDim] = {false, false, false, false};
    int64_t size[kMaxDim] = {0, 0, 0, 0};
    double lo[kMaxDim] = {0, 0, 0, 0};
    double hi[kMaxDim] = {0, 0, 0, 0};
    const double* coords[kMaxDim] = {nullptr, nullptr, nullptr, nullptr};
};

struct TableModel {
    int dim = 0;
    int order = 0;
    AxisModel axis[kMaxDim];
    int64_t total = 0;
};

// Builds knots and factors. Returns an empty string on success, else the
// reason (invalid sizes, non-monotonic coordinates, ...).
std::string build_model(const TableSpec& spec, TableModel& out, bool need_solver = true);

// Solves A x = b in place in FP64 with a factor in row layout (host).
void line_factor_solve(const LineFactor& f, double* x);

// Predicted relative error of an FP32 control-point solve: about FP32
// epsilon times the sum of the per-axis condition estimates.
double fp32_solve_error_estimate(const TableModel& m);

// Knot-span hint of the reference (Interpolation.hpp:277-295); the span that
// evaluation finds does not depend on it, it only seeds the search.
int64_t knot_hint(const AxisModel& ax, int order, double x);

// Cox-de Boor basis of BSpline::base_spline_value (BSpline.hpp:83-111):
// out[0..order], right-aligned when spline_order < order.
void base_spline_value(const double* knots, int64_t seg, double x, int order, int spline_order,
                       double* out);

}  // namespace intp_gb300
