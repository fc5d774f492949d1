// C-ABI driver around the reference library's own headers (12ff54e/
// BSplineInterpolation, src/include/*.hpp), compiled in place by
// oracle/build_ref.sh into oracle/_ref/. TEST INFRASTRUCTURE ONLY: it lets the
// tests pin the C restatement (intp_oracle.c) against the reference itself and
// lets the golden-fixture script record reference outputs. Nothing in the
// product loads it, and it is never built where the reference is absent.
//
// Instantiated for D in {1,2,3}, O in {0..7}. Non-uniform axes (iterator-pair
// ranges) are available for D <= 2 in every per-axis combination, and for
// D == 3 only with all axes uniform.
#include <Interpolation.hpp>
#include <BandLU.hpp>
#include <BandMatrix.hpp>

#include <array>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace {

thread_local std::string g_err;
// seconds spent in the last InterpolationFunction constructor (knots, factors
// and the control-point solve), without the driver's own mesh copy
thread_local double g_build_seconds = 0.0;

struct Handle {
    virtual ~Handle() = default;
    virtual int dim() const = 0;
    virtual void eval(const double* c, int64_t n, double* out, int nthreads) const = 0;
    virtual void eval_deriv(const double* c, int64_t n, const int* k, int nk, double* out,
                            int nthreads) const = 0;
    virtual int64_t nknots(int axis) const = 0;
    virtual void knots(int axis, double* out) const = 0;
    virtual void range(int axis, double* lo, double* hi) const = 0;
    virtual void locate(const double* c, int64_t n, int64_t* cells, double* wrapped) const = 0;
    virtual int64_t nctrl() const = 0;
    virtual void ctrl(double* out) const = 0;
    virtual int at_check(const double* c) const = 0;
    // outputs as a user of the reference computes them: operator() for a row
    // of all-zero orders, derivative() otherwise
    virtual void eval_user(const double* c, int64_t n, const int* k, int nk, double* out, int nthreads) const {
        eval_deriv(c, n, k, nk, out, nthreads);
    }
};

template <typename F>
void parallel_for(int64_t n, int nthreads, F&& f) {
    if (nthreads <= 1 || n < 1024) {
        f(int64_t{0}, n);
        return;
    }
    std::vector<std::thread> th;
    for (int k = 0; k < nthreads; ++k)
        th.emplace_back([&, k] { f(n * k / nthreads, n * (k + 1) / nthreads); });
    for (auto& t : th) t.join();
}

template <std::size_t D, std::size_t O>
struct FnHandle : Handle {
    using Fn = intp::InterpolationFunction<double, D, O>;
    Fn fn;
    explicit FnHandle(Fn&& f) : fn(std::move(f)) {}
    int dim() const override { return (int)D; }
    void eval(const double* c, int64_t n, double* out, int nthreads) const override {
        parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
            for (int64_t p = b; p < e; ++p) {
                std::array<double, D> x;
                for (std::size_t d = 0; d < D; ++d) x[d] = c[p * (int64_t)D + (int64_t)d];
                out[p] = fn(x);
            }
        });
    }
    void eval_deriv(const double* c, int64_t n, const int* k, int nk, double* out,
                    int nthreads) const override {
        parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
            for (int64_t p = b; p < e; ++p) {
                std::array<double, D> x;
                for (std::size_t d = 0; d < D; ++d) x[d] = c[p * (int64_t)D + (int64_t)d];
                for (int r = 0; r < nk; ++r) {
                    std::array<std::size_t, D> kk;
                    for (std::size_t d = 0; d < D; ++d) kk[d] = (std::size_t)k[r * (int)D + (int)d];
                    out[p * nk + r] = fn.derivative(x, kk);
                }
            }
        });
    }
    void eval_user(const double* c, int64_t n, const int* k, int nk, double* out,
                   int nthreads) const override {
        parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
            std::array<std::size_t, D> kk[16];
            bool value[16];
            for (int r = 0; r < nk && r < 16; ++r) {
                value[r] = true;
                for (std::size_t d = 0; d < D; ++d) {
                    kk[r][d] = (std::size_t)k[r * (int)D + (int)d];
                    value[r] = value[r] && kk[r][d] == 0;
                }
            }
            for (int64_t p = b; p < e; ++p) {
                std::array<double, D> x;
                for (std::size_t d = 0; d < D; ++d) x[d] = c[p * (int64_t)D + (int64_t)d];
                for (int r = 0; r < nk && r < 16; ++r)
                    out[p * nk + r] = value[r] ? fn(x) : fn.derivative(x, kk[r]);
            }
        });
    }
    int64_t nknots(int axis) const override { return (int64_t)fn.spline().knots_num(axis); }
    void knots(int axis, double* out) const override {
        auto b = fn.spline().knots_begin(axis), e = fn.spline().knots_end(axis);
        std::size_t i = 0;
        for (auto it = b; it != e; ++it) out[i++] = *it;
    }
    void range(int axis, double* lo, double* hi) const override {
        *lo = fn.range(axis).first;
        *hi = fn.range(axis).second;
    }
    void locate(const double* c, int64_t n, int64_t* cells, double* wrapped) const override {
        // The knot span does not depend on the hint (any in-range hint gives
        // the same span), so hint O is used.
        const auto& sp = fn.spline();
        for (int64_t p = 0; p < n; ++p)
            for (std::size_t d = 0; d < D; ++d) {
                double x = c[p * (int64_t)D + (int64_t)d];
                auto it = sp.get_knot_iter(d, x, O);
                cells[p * (int64_t)D + (int64_t)d] = (int64_t)(it - sp.knots_begin(d));
                if (wrapped) wrapped[p * (int64_t)D + (int64_t)d] = x;
            }
    }
    int64_t nctrl() const override { return (int64_t)fn.spline().control_points().size(); }
    void ctrl(double* out) const override {
        const auto& cp = fn.spline().control_points();
        std::size_t i = 0;
        for (auto it = cp.begin(); it != cp.end(); ++it) out[i++] = *it;
    }
    int at_check(const double* c) const override {
        std::array<double, D> x;
        for (std::size_t d = 0; d < D; ++d) x[d] = c[d];
        try {
            (void)fn.at(x);
            return 1;
        } catch (const std::domain_error&) {
            return 0;
        }
    }
};

using Range = std::pair<double, double>;
using Iter = std::pair<const double*, const double*>;

struct AxisArg {
    bool uniform;
    Range r;
    Iter it;
};

template <std::size_t D>
intp::Mesh<double, D> make_mesh(const int64_t* sizes, const double* values) {
    std::array<std::size_t, D> dims;
    for (std::size_t d = 0; d < D; ++d) dims[d] = (std::size_t)sizes[d];
    intp::Mesh<double, D> m{intp::MeshDimension<D>(dims)};
    std::size_t total = 1;
    for (auto s : dims) total *= s;
    for (std::size_t i = 0; i < total; ++i) m(m.dimension().dimwise_indices(i)) = values[i];
    return m;
}

template <std::size_t D, std::size_t O, typename... A>
Handle* construct(const std::array<bool, D>& per, const intp::Mesh<double, D>& m, A... a) {
    const auto t0 = std::chrono::steady_clock::now();
    intp::InterpolationFunction<double, D, O> fn(per, m, a...);
    g_build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return new FnHandle<D, O>(std::move(fn));
}

template <std::size_t O>
Handle* build1(const bool* per, const int64_t* sizes, const double* v, const AxisArg* ax) {
    auto m = make_mesh<1>(sizes, v);
    std::array<bool, 1> p{per[0]};
    if (ax[0].uniform) return construct<1, O>(p, m, ax[0].r);
    return construct<1, O>(p, m, ax[0].it);
}

template <std::size_t O>
Handle* build2(const bool* per, const int64_t* sizes, const double* v, const AxisArg* ax) {
    auto m = make_mesh<2>(sizes, v);
    std::array<bool, 2> p{per[0], per[1]};
    if (ax[0].uniform && ax[1].uniform) return construct<2, O>(p, m, ax[0].r, ax[1].r);
    if (ax[0].uniform && !ax[1].uniform) return construct<2, O>(p, m, ax[0].r, ax[1].it);
    if (!ax[0].uniform && ax[1].uniform) return construct<2, O>(p, m, ax[0].it, ax[1].r);
    return construct<2, O>(p, m, ax[0].it, ax[1].it);
}

template <std::size_t O>
Handle* build3(const bool* per, const int64_t* sizes, const double* v, const AxisArg* ax) {
    auto m = make_mesh<3>(sizes, v);
    std::array<bool, 3> p{per[0], per[1], per[2]};
    if (ax[0].uniform && ax[1].uniform && ax[2].uniform)
        return construct<3, O>(p, m, ax[0].r, ax[1].r, ax[2].r);
    throw std::invalid_argument("3D non-uniform axes are not instantiated in the driver");
}

template <std::size_t O>
Handle* build_o(int dim, const bool* per, const int64_t* sizes, const double* v,
                const AxisArg* ax) {
    switch (dim) {
        case 1: return build1<O>(per, sizes, v, ax);
        case 2: return build2<O>(per, sizes, v, ax);
        case 3: return build3<O>(per, sizes, v, ax);
    }
    throw std::invalid_argument("dimension not instantiated");
}

// Bare BSpline from explicit knots (test/src/bspline-test.cpp usage), O = 3.
template <std::size_t D>
struct SplineHandle : Handle {
    using Sp = intp::BSpline<double, D, 3>;
    std::unique_ptr<Sp> sp;
    int dim() const override { return (int)D; }
    void eval(const double* c, int64_t n, double* out, int) const override {
        for (int64_t p = 0; p < n; ++p) {
            std::array<double, D> x;
            for (std::size_t d = 0; d < D; ++d) x[d] = c[p * (int64_t)D + (int64_t)d];
            out[p] = (*sp)(x);
        }
    }
    void eval_deriv(const double* c, int64_t n, const int* k, int nk, double* out,
                    int) const override {
        for (int64_t p = 0; p < n; ++p)
            for (int r = 0; r < nk; ++r) {
                std::array<std::pair<double, std::size_t>, D> a;
                for (std::size_t d = 0; d < D; ++d)
                    a[d] = {c[p * (int64_t)D + (int64_t)d], (std::size_t)k[r * (int)D + (int)d]};
                out[p * nk + r] = sp->derivative_at(a);
            }
    }
    int64_t nknots(int axis) const override { return (int64_t)sp->knots_num(axis); }
    void knots(int axis, double* out) const override {
        std::size_t i = 0;
        for (auto it = sp->knots_begin(axis); it != sp->knots_end(axis); ++it) out[i++] = *it;
    }
    void range(int axis, double* lo, double* hi) const override {
        *lo = sp->range(axis).first;
        *hi = sp->range(axis).second;
    }
    void locate(const double*, int64_t, int64_t*, double*) const override {}
    int64_t nctrl() const override { return 0; }
    void ctrl(double*) const override {}
    int at_check(const double*) const override { return 1; }
};

template <std::size_t D, std::size_t... I>
Handle* make_spline(std::index_sequence<I...>, const bool* per, const int64_t* ncp,
                    const double* const* knots, const int64_t* nk, const double* ctrl) {
    using Sp = intp::BSpline<double, D, 3>;
    typename Sp::ControlPointContainer cp{intp::MeshDimension<D>((std::size_t)ncp[I]...)};
    std::size_t total = 1;
    for (std::size_t d = 0; d < D; ++d) total *= (std::size_t)ncp[d];
    for (std::size_t i = 0; i < total; ++i) cp(cp.dimension().dimwise_indices(i)) = ctrl[i];
    std::array<bool, D> p{per[I]...};
    auto h = new SplineHandle<D>();
    h->sp.reset(new Sp(p, cp, std::make_pair(knots[I], knots[I] + nk[I])...));
    return h;
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

void* ref_create(int dim, int order, const int* periodic, const int64_t* sizes,
                 const double* lo, const double* hi, const double* const* coords,
                 const double* values) {
    try {
        bool per[3] = {false, false, false};
        AxisArg ax[3];
        for (int d = 0; d < dim && d < 3; ++d) {
            per[d] = periodic && periodic[d];
            ax[d].uniform = !(coords && coords[d]);
            ax[d].r = {lo ? lo[d] : 0.0, hi ? hi[d] : 0.0};
            if (!ax[d].uniform) {
                const int64_t n = sizes[d] + (per[d] ? 1 : 0);
                ax[d].it = {coords[d], coords[d] + n};
            }
        }
        switch (order) {
            case 0: return build_o<0>(dim, per, sizes, values, ax);
            case 1: return build_o<1>(dim, per, sizes, values, ax);
            case 2: return build_o<2>(dim, per, sizes, values, ax);
            case 3: return build_o<3>(dim, per, sizes, values, ax);
            case 4: return build_o<4>(dim, per, sizes, values, ax);
            case 5: return build_o<5>(dim, per, sizes, values, ax);
            case 6: return build_o<6>(dim, per, sizes, values, ax);
            case 7: return build_o<7>(dim, per, sizes, values, ax);
        }
        g_err = "order not instantiated";
    } catch (const std::exception& e) {
        g_err = e.what();
    }
    return nullptr;
}

void* ref_create_bspline(int dim, const int* periodic, const int64_t* ncp,
                         const double* const* knots, const int64_t* nknots,
                         const double* ctrl) {
    try {
        bool per[3] = {false, false, false};
        for (int d = 0; d < dim && d < 3; ++d) per[d] = periodic && periodic[d];
        switch (dim) {
            case 1: return make_spline<1>(std::make_index_sequence<1>{}, per, ncp, knots, nknots, ctrl);
            case 2: return make_spline<2>(std::make_index_sequence<2>{}, per, ncp, knots, nknots, ctrl);
            case 3: return make_spline<3>(std::make_index_sequence<3>{}, per, ncp, knots, nknots, ctrl);
        }
        g_err = "dimension not instantiated";
    } catch (const std::exception& e) {
        g_err = e.what();
    }
    return nullptr;
}

void ref_free(void* h) { delete static_cast<Handle*>(h); }

void ref_eval(void* h, const double* c, int64_t n, double* out, int nthreads) {
    static_cast<Handle*>(h)->eval(c, n, out, nthreads);
}

void ref_eval_deriv(void* h, const double* c, int64_t n, const int* k, int nk, double* out,
                    int nthreads) {
    static_cast<Handle*>(h)->eval_deriv(c, n, k, nk, out, nthreads);
}

void ref_eval_user(void* h, const double* c, int64_t n, const int* k, int nk, double* out, int nthreads) {
    static_cast<Handle*>(h)->eval_user(c, n, k, nk, out, nthreads);
}

double ref_last_build_seconds() { return g_build_seconds; }

int64_t ref_num_knots(void* h, int axis) { return static_cast<Handle*>(h)->nknots(axis); }
void ref_knots(void* h, int axis, double* out) { static_cast<Handle*>(h)->knots(axis, out); }
void ref_range(void* h, int axis, double* lo, double* hi) {
    static_cast<Handle*>(h)->range(axis, lo, hi);
}
void ref_locate(void* h, const double* c, int64_t n, int64_t* cells, double* wrapped) {
    static_cast<Handle*>(h)->locate(c, n, cells, wrapped);
}
int64_t ref_num_ctrl(void* h) { return static_cast<Handle*>(h)->nctrl(); }
void ref_ctrl(void* h, double* out) { static_cast<Handle*>(h)->ctrl(out); }
int ref_at_check(void* h, const double* c) { return static_cast<Handle*>(h)->at_check(c); }

// BandLU on a dense description (test/src/band-matrix-and-solver-test.cpp).
int ref_band_solve_dense(int64_t n, int p, int q, int cyclic, const double* a, double* b) {
    try {
        const std::size_t N = (std::size_t)n, P = (std::size_t)p, Q = (std::size_t)q;
        if (!cyclic) {
            intp::BandMatrix<double> m{N, P, Q};
            for (std::size_t i = 0; i < N; ++i)
                for (std::size_t j = 0; j < N; ++j)
                    if (j + P >= i && i + Q >= j) m(i, j) = a[i * N + j];
            intp::BandLU<intp::BandMatrix<double>> lu{std::move(m)};
            std::vector<double> x(b, b + N);
            lu.solve_in_place(x.data());
            std::memcpy(b, x.data(), N * sizeof(double));
        } else {
            intp::ExtendedBandMatrix<double> m{N, P, Q};
            for (std::size_t i = 0; i < N; ++i)
                for (std::size_t j = 0; j < N; ++j) {
                    const bool in_main = j + P >= i && i + Q >= j;
                    const bool in_side = (j >= std::max(N - P, i + Q + 1)) ||
                                         (i >= std::max(N - Q, j + P + 1));
                    if (in_main || in_side) m(i, j) = a[i * N + j];
                }
            intp::BandLU<intp::ExtendedBandMatrix<double>> lu{std::move(m)};
            std::vector<double> x(b, b + N);
            lu.solve_in_place(x.data());
            std::memcpy(b, x.data(), N * sizeof(double));
        }
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

}  // extern "C"
