// Host-side table model: knots, collocation matrices, band LU factors.
// Arithmetic is written in the reference's operation order so knot vectors are
// bit-identical to the reference's (cell indices depend on them exactly); this
// translation unit is compiled without floating-point contraction.
#include "spline_model.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace intp_gb300 {

void BandStore::reset(int64_t n_, int64_t p_, int64_t q_, bool cyclic_) {
    n = n_;
    p = p_;
    q = q_;
    cyclic = cyclic_;
    band.assign(static_cast<size_t>(n * (1 + p + q)), 0.0);
    right.clear();
    bottom.clear();
    if (cyclic) {
        right.assign(static_cast<size_t>(std::max<int64_t>(n - q - 1, 0) * p + 1), 0.0);
        bottom.assign(static_cast<size_t>(std::max<int64_t>(n - p - 1, 0) * q + 1), 0.0);
    }
}

void BandStore::factorize() {
    if (!cyclic) {
        // BandLU<BandMatrix>::compute_impl, BandLU.hpp:103-118
        for (int64_t k = 0; k + 1 < n; ++k) {
            const int64_t ie = std::min(k + p + 1, n), je = std::min(k + q + 1, n);
            for (int64_t i = k + 1; i < ie; ++i) at_main(i, k) /= at_main(k, k);
            for (int64_t j = k + 1; j < je; ++j)
                for (int64_t i = k + 1; i < ie; ++i) at_main(i, j) -= at_main(i, k) * at_main(k, j);
        }
        return;
    }
    // BandLU<ExtendedBandMatrix>::compute_impl, BandLU.hpp:159-213
    for (int64_t k = 0; k + 1 < n; ++k) {
        const int64_t ie = std::min(k + p + 1, n), je = std::min(k + q + 1, n);
        const int64_t side_i0 = std::max(n - q, k + p + 1), side_j0 = std::max(n - p, k + q + 1);
        for (int64_t i = k + 1; i < ie; ++i) at_main(i, k) /= at_main(k, k);
        for (int64_t i = side_i0; i < n; ++i) at_side(i, k) /= at_main(k, k);
        for (int64_t j = k + 1; j < je; ++j)
            for (int64_t i = k + 1; i < ie; ++i) at_main(i, j) -= at_main(i, k) * at_main(k, j);
        for (int64_t i = k + 1; i < ie; ++i)
            for (int64_t j = side_j0; j < n; ++j) at(i, j) -= at_main(i, k) * at_side(k, j);
        for (int64_t j = k + 1; j < je; ++j)
            for (int64_t i = side_i0; i < n; ++i) at(i, j) -= at_side(i, k) * at_main(k, j);
        if (k < std::max(n - p - 1, n - q - 1))
            for (int64_t i = side_i0; i < n; ++i)
                for (int64_t j = side_j0; j < n; ++j) at_main(i, j) -= at_side(i, k) * at_side(k, j);
    }
}

void BandStore::multiply(const double* x, double* y) const {
    for (int64_t i = 0; i < n; ++i) {
        double s = 0.0;
        for (int64_t j = std::max<int64_t>(i - p, 0); j < std::min(i + q + 1, n); ++j)
            s += at_main(i, j) * x[j];
        if (cyclic && i < n - q - 1)
            for (int64_t j = std::max(n - p, i + q + 1); j < n; ++j) s += at_side(i, j) * x[j];
        y[i] = s;
    }
    if (cyclic)
        for (int64_t j = 0; j < n - p - 1; ++j)
            for (int64_t i = std::max(n - q, j + p + 1); i < n; ++i) y[i] += at_side(i, j) * x[j];
}

void base_spline_value(const double* t, int64_t seg, double x, int order, int spline_order,
                       double* out) {
    for (int k = 0; k <= order; ++k) out[k] = 0.0;
    out[order] = 1.0;
    for (int i = 1; i <= spline_order; ++i) {
        const int b = order - i;
        for (int j = 0; j <= i; ++j) {
            const int64_t l = seg - (i - j), r = seg + j + 1;
            const double left = j == 0 ? 0.0 : out[b + j] * (x - t[l]) / (t[r - 1] - t[l]);
            const double right = b + j == order ? 0.0 : out[b + j + 1] * (t[r] - x) / (t[r] - t[l + 1]);
            out[b + j] = left + right;
        }
    }
}

int64_t knot_hint(const AxisModel& ax, int order, double x) {
    if (!ax.uniform) return order;
    const int64_t cap = static_cast<int64_t>(ax.knots.size()) - order - 2;
    double v = (x - ax.range_lo) / ax.dx - (ax.periodic ? 1.0 : 0.5 * static_cast<double>(order + 1));
    if (!(v > 0.0)) v = 0.0;
    v = std::ceil(v);
    if (v > static_cast<double>(cap)) return cap;
    return std::min(cap, static_cast<int64_t>(v) + order);
}

LineFactor line_factor_from(const BandStore& lu) {
    LineFactor f;
    const int64_t n = lu.n, p = lu.p, q = lu.q;
    f.n = n;
    f.p = static_cast<int>(p);
    f.q = static_cast<int>(q);
    f.cyclic = lu.cyclic;
    f.lower.assign(static_cast<size_t>(n * std::max<int64_t>(p, 1)), 0.0);
    f.upper.assign(static_cast<size_t>(n * std::max<int64_t>(q, 1)), 0.0);
    f.dinv.assign(static_cast<size_t>(n), 0.0);
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t k = 0; k < p; ++k) {
            const int64_t j = i - p + k;
            if (j >= 0) f.lower[i * p + k] = lu.at_main(i, j);
        }
        for (int64_t k = 0; k < q; ++k) {
            const int64_t j = i + 1 + k;
            if (j < n) f.upper[i * q + k] = lu.at_main(i, j);
        }
        f.dinv[i] = 1.0 / lu.at_main(i, i);
    }
    if (lu.cyclic) {
        f.bottom.assign(static_cast<size_t>(std::max<int64_t>(q, 1) * n), 0.0);
        f.right.assign(static_cast<size_t>(std::max<int64_t>(p, 1) * n), 0.0);
        for (int64_t r = 0; r < q; ++r) {
            const int64_t i = n - q + r;
            for (int64_t j = 0; j < n - p - 1; ++j)
                if (i >= j + p + 1) f.bottom[r * n + j] = lu.at_side(i, j);
        }
        for (int64_t r = 0; r < p; ++r) {
            const int64_t j = n - p + r;
            for (int64_t i = 0; i < j - q; ++i) f.right[r * n + i] = lu.at_side(i, j);
        }
    }
    // the longest run of rows identical to its first row (bitwise): band,
    // dinv and, on a cyclic factor, the side-band entries of the row (these
    // decay away from the corners and reach exactly 0); once for the FP64
    // values and once for their FP32 roundings
    auto longest_run = [&](auto tag, int64_t& out_lo, int64_t& out_hi) {
        using T = decltype(tag);
        auto eq = [](double a, double b) {
            T x, y;
            if constexpr (sizeof(T) == 4) {
                x = factor_f32(a);
                y = factor_f32(b);
            } else {
                x = a;
                y = b;
            }
            return std::memcmp(&x, &y, sizeof(T)) == 0;
        };
        auto same = [&](int64_t a, int64_t b) {
            if (!eq(f.dinv[a], f.dinv[b])) return false;
            for (int64_t k = 0; k < p; ++k)
                if (!eq(f.lower[a * p + k], f.lower[b * p + k])) return false;
            for (int64_t k = 0; k < q; ++k)
                if (!eq(f.upper[a * q + k], f.upper[b * q + k])) return false;
            if (f.cyclic) {
                for (int64_t r = 0; r < q; ++r)
                    if (!eq(f.bottom[r * n + a], f.bottom[r * n + b])) return false;
                for (int64_t r = 0; r < p; ++r)
                    if (!eq(f.right[r * n + a], f.right[r * n + b])) return false;
            }
            return true;
        };
        int64_t best_lo = 0, best_hi = 0, lo = 0;
        for (int64_t i = 1; i <= n; ++i) {
            if (i == n || !same(lo, i)) {
                if (i - lo > best_hi - best_lo) {
                    best_lo = lo;
                    best_hi = i;
                }
                lo = i;
            }
        }
        out_lo = out_hi = 0;
        if (best_hi - best_lo >= 2) {
            out_lo = best_lo;
            out_hi = best_hi;
        }
    };
    if (n > 0) {
        longest_run(double{}, f.const_lo, f.const_hi);
        longest_run(float{}, f.const_lo32, f.const_hi32);
    }
    if (f.cyclic) {
        // the first row from which every later side-band sum entry is zero
        const int64_t nb = n - p - 1;
        f.zside = f.zside32 = nb > 0 ? nb : 0;
        bool nz64 = false, nz32 = false;
        for (int64_t i = nb - 1; i >= 0 && !(nz64 && nz32); --i)
            for (int64_t r = 0; r < q; ++r) {
                const double v = f.bottom[r * n + i];
                if (!nz64 && v != 0.0) {
                    nz64 = true;
                    f.zside = i + 1;
                }
                if (!nz32 && factor_f32(v) != 0.0f) {
                    nz32 = true;
                    f.zside32 = i + 1;
                }
            }
        if (!nz64) f.zside = 0;
        if (!nz32) f.zside32 = 0;
    }
    return f;
}

void line_factor_solve(const LineFactor& f, double* x) {
    const int64_t n = f.n, p = f.p, q = f.q;
    std::vector<double> acc(static_cast<size_t>(q > 0 ? q : 1), 0.0);
    if (f.cyclic)
        for (int64_t r = 0; r < q; ++r) acc[r] = x[n - q + r];
    for (int64_t i = 0; i < n; ++i) {
        double v = (f.cyclic && i >= n - q) ? acc[i - (n - q)] : x[i];
        for (int64_t k = 0; k < p; ++k)
            if (i - p + k >= 0) v -= f.lower[i * p + k] * x[i - p + k];
        if (f.cyclic && i < n - p - 1)
            for (int64_t r = 0; r < q; ++r) acc[r] -= f.bottom[r * n + i] * v;
        x[i] = v;
    }
    for (int64_t i = n - 1; i >= 0; --i) {
        double v = x[i];
        if (f.cyclic)
            for (int64_t r = p - 1; r >= 0; --r)
                if (n - p + r > i + q) v -= f.right[r * n + i] * x[n - p + r];
        for (int64_t k = q - 1; k >= 0; --k)
            if (i + 1 + k < n) v -= f.upper[i * q + k] * x[i + 1 + k];
        x[i] = v * f.dinv[i];
    }
}

double fp32_solve_error_estimate(const TableModel& m) {
    double s = 0.0;
    for (int d = 0; d < m.dim; ++d) s += m.axis[d].cond_est;
    return 6.0e-8 * s;
}

namespace {

// Condition estimate of a collocation matrix. B-spline collocation matrices
// are totally positive, so the inverse has a checkerboard sign pattern and
// ||A^-1||_inf = ||A^-1 s||_inf for the alternating vector s (one solve);
// for the cyclic (periodic) matrices the same solve gives the estimate.
double condition_estimate(const AxisModel& ax) {
    const int64_t n = ax.n;
    std::vector<double> x(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) x[i] = (i % 2) ? -1.0 : 1.0;
    line_factor_solve(ax.factor, x.data());
    double inv = 0.0, a = 0.0;
    for (int64_t i = 0; i < n; ++i) inv = std::max(inv, std::fabs(x[i]));
    for (int64_t i = 0; i < n; ++i) {
        double row = 0.0;
        for (int w = 0; w < ax.stencil.width; ++w) row += std::fabs(ax.stencil.val[i * ax.stencil.width + w]);
        a = std::max(a, row);
    }
    return std::isfinite(a * inv) ? a * inv : 1e300;
}

// Uniform knots, Interpolation.hpp:322-362 (NO_DUMMY: n = size + periodic).
std::string uniform_knots(AxisModel& ax, int order, double x0, double x1) {
    const int64_t n = ax.n + (ax.periodic ? 1 : 0);
    if (n < 2) return "a uniform axis needs at least 2 points";
    if (!(x1 > x0)) return "an axis range must be increasing";
    ax.uniform = true;
    ax.dx = (x1 - x0) / static_cast<double>(n - 1);
    const int64_t extra = ax.periodic ? 2 * order + (1 - order % 2) : order + 1;
    const int64_t sz = n + extra;
    ax.knots.assign(static_cast<size_t>(sz), x0);
    const double half_extra = 0.5 * static_cast<double>(extra);
    const int64_t first = ax.periodic ? 0 : order + 1;
    const int64_t last = ax.periodic ? sz : sz - order - 1;
    for (int64_t i = first; i < last; ++i)
        ax.knots[i] = x0 + (static_cast<double>(i) - half_extra) * ax.dx;
    if (!ax.periodic)
        for (int64_t i = sz - order - 1; i < sz; ++i) ax.knots[i] = x1;
    ax.range_lo = ax.knots[order];
    ax.range_hi = ax.knots[sz - order - (2 - order % 2)];  // BSpline.hpp:222-227
    return {};
}

// Non-uniform knots, Interpolation.hpp:365-464.
std::string nonuniform_knots(AxisModel& ax, int order, const double* c) {
    const int64_t n = ax.n + (ax.periodic ? 1 : 0);
    if (!ax.periodic && order == 0) return "a non-uniform non-periodic axis needs order >= 1";
    if (n < 2) return "a non-uniform axis needs at least 2 coordinates";
    ax.uniform = false;
    ax.dx = 0.0;
    const int64_t sz = ax.periodic ? n + 2 * order + (1 - order % 2) : n + order + 1;
    std::vector<double> xs(static_cast<size_t>(sz), 0.0);
    std::vector<double>& in = ax.input_coords;
    in.clear();
    in.reserve(static_cast<size_t>(n));
    if (ax.periodic) {
        // knots are the samples, shifted half a cell for even orders
        in.push_back(c[0]);
        for (int64_t i = order + 1; i < order + n; ++i) {
            const double present = c[i - order];
            xs[i] = order % 2 == 0 ? 0.5 * (in.back() + present) : present;
            in.push_back(present);
        }
        const double period = in.back() - in.front();
        for (int64_t i = 0; i < order + 1; ++i) {
            xs[i] = xs[n + i - 1] - period;
            xs[sz - i - 1] = xs[sz - i - n] + period;
        }
    } else {
        // interior knots: moving averages of `order` consecutive samples
        for (int64_t i = 0; i < order + 1; ++i) xs[i] = c[0];
        in.push_back(c[0]);
        double window = 0.0;
        for (int64_t i = 1; i < order; ++i) {
            in.push_back(c[i]);
            window += in[i];
        }
        for (int64_t i = order + 1; i < n; ++i) {
            in.push_back(c[i - 1]);
            window += in[i - 1];
            xs[i] = window / static_cast<double>(order);
            window -= in[i - order];
        }
        for (int64_t i = n; i < n + order + 1; ++i) xs[i] = c[n - 1];
        in.push_back(c[n - 1]);
    }
    for (size_t i = 0; i + 1 < in.size(); ++i)
        if (!(in[i + 1] > in[i])) return "given coordinate is not monotonically increasing";
    ax.knots = std::move(xs);
    ax.range_lo = ax.knots[order];
    ax.range_hi = ax.knots[sz - order - (2 - order % 2)];
    return {};
}

// Collocation matrix of one axis and its factor,
// InterpolationTemplate.hpp:254-446 (C++17 branch).
std::string build_axis_solver(AxisModel& ax, int order) {
    const int64_t n = ax.n;
    const int64_t bw = ax.periodic ? order / 2 : (order == 0 ? 0 : order - 1);
    if (ax.periodic && n < 2 * bw + 1) return "periodic axis too short for this order";
    ax.colloc.reset(n, bw, bw, ax.periodic);
    const double* t = ax.knots.data();
    const int64_t knot_num = static_cast<int64_t>(ax.knots.size());
    double base[kMaxOrder + 1];
    if (ax.periodic && ax.uniform)
        base_spline_value(t, order, t[order] + static_cast<double>(1 - order % 2) * ax.dx * 0.5, order,
                          order, base);
    for (int64_t i = 0; i < n; ++i) {
        if (!ax.periodic && (i == 0 || i == n - 1)) {
            ax.colloc.at(i, i) = 1.0;
            continue;
        }
        int64_t knot_ind = 0;
        const bool internal = i > order / 2 && i < n - order / 2 - 1;
        if (ax.uniform) {
            knot_ind = ax.periodic ? i + order
                                   : std::min(knot_num - order - 2, i > order / 2 ? i + (order + 1) / 2 : int64_t(order));
            if (!ax.periodic && (knot_ind <= 2 * order + 1 || knot_ind >= knot_num - 2 * order - 2)) {
                // near the clamped ends the basis differs; elsewhere the last
                // computed one is reused (:347-360)
                const double x = ax.range_lo + static_cast<double>(i) * ax.dx;
                base_spline_value(t, knot_ind, x, order, order, base);
            }
        } else {
            const double x = ax.input_coords[i];
            int64_t it;
            if (ax.periodic) {
                it = i + order;
            } else if (i == 0) {
                it = order;
            } else if (i == static_cast<int64_t>(ax.input_coords.size()) - 1) {
                it = knot_num - (order + 2);
            } else {
                const int64_t hint = i + 1, last = std::min(knot_num - order - 1, i + order);
                if (t[hint] <= x && t[hint + 1] > x) {
                    it = hint;
                } else {
                    it = std::upper_bound(t + order + 1, t + last + 1, x) - t - 1;
                }
            }
            knot_ind = it;
            base_spline_value(t, it, x, order, order, base);
        }
        const int64_t s_num = ax.periodic ? (order | 1)
                              : order == 1 ? 1
                              : (ax.uniform && internal) ? (order | 1)
                                                         : order + 1;
        for (int64_t j = 0; j < s_num; ++j) {
            const int64_t row = (i + (ax.periodic ? bw : 0)) % n;
            const int64_t col = (knot_ind - order + j) % n;
            ax.colloc.at(row, col) = base[j];
        }
    }
    ax.lu = ax.colloc;
    ax.lu.factorize();

    ax.factor = line_factor_from(ax.lu);

    const int64_t p = bw, q = bw;
    // collocation rows as a stencil (for FP64 residuals): row i couples
    // columns i-p .. i+q, taken cyclically on a periodic axis (the corner
    // blocks of the cyclic matrix hold exactly the wrapped neighbours)
    RowStencil& s = ax.stencil;
    s.n = n;
    s.width = static_cast<int>(1 + p + q);
    s.col.assign(static_cast<size_t>(n * s.width), 0);
    s.val.assign(static_cast<size_t>(n * s.width), 0.0);
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t k = -p; k <= q; ++k) {
            const int64_t w = i * s.width + (k + p);
            int64_t j = i + k;
            if (ax.periodic) {
                j = ((j % n) + n) % n;
            } else if (j < 0 || j >= n) {
                s.col[w] = i;
                continue;
            }
            s.col[w] = j;
            s.val[w] = ax.colloc.at(i, j);
        }
    }
    ax.cond_est = condition_estimate(ax);
    return {};
}

}  // namespace

std::string build_model(const TableSpec& spec, TableModel& out, bool need_solver) {
    if (spec.dim < 1 || spec.dim > kMaxDim) return "dimension must be in [1, 4]";
    if (spec.order < 0 || spec.order > kMaxOrder) return "order must be in [0, 7]";
    out = TableModel{};
    out.dim = spec.dim;
    out.order = spec.order;
    out.total = 1;
    for (int d = 0; d < spec.dim; ++d) {
        AxisModel& ax = out.axis[d];
        ax.n = spec.size[d];
        ax.periodic = spec.periodic[d];
        if (ax.n < 1) return "every axis needs at least one sample";
        if (!ax.periodic && ax.n < static_cast<int64_t>(spec.order) + 1)
            return "a non-periodic axis needs at least order+1 samples";
        out.total *= ax.n;
        std::string err = spec.coords[d] ? nonuniform_knots(ax, spec.order, spec.coords[d])
                                         : uniform_knots(ax, spec.order, spec.lo[d], spec.hi[d]);
        if (!err.empty()) return err;
        if (need_solver) {
            err = build_axis_solver(ax, spec.order);
            if (!err.empty()) return err;
        }
    }
    return {};
}

}  // namespace intp_gb300
