// Exercises the header-only C++ drop-in (include/intp/Interpolation.hpp) the
// way the reference's own tests use the reference (test/src/
// interpolation-test.cpp): InterpolationFunction<double, D, O> built from a
// Mesh with uniform (min, max) or iterator-pair ranges per axis, evaluated
// point by point with operator() / derivative_at, and in batches.
//
// Reads cases from stdin (one per line):
//   name dim order periodic[dim] size[dim] axis[dim] nvalues values... npts points... nderiv derivs...
// where axis = "U lo hi" or "N count coords..." (doubles in hex). Prints per
// case "name" then the single-point results and the batch results, in hex.
#include <intp/Interpolation.hpp>

#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <array>
#include <vector>

struct Case {
    std::string name;
    int dim = 0, order = 0;
    std::vector<int> periodic;
    std::vector<long long> size;
    std::vector<int> uniform;
    std::vector<double> lo, hi;
    std::vector<std::vector<double>> coords;
    std::vector<double> values, points;
    std::vector<int32_t> derivs;
    int nderiv = 0;
};

static bool read_double(double& v) { return std::scanf("%la", &v) == 1; }

static bool read_case(Case& c) {
    char buf[256];
    if (std::scanf("%255s", buf) != 1) return false;
    c.name = buf;
    if (std::scanf("%d %d", &c.dim, &c.order) != 2) return false;
    c.periodic.resize(c.dim);
    c.size.resize(c.dim);
    c.uniform.resize(c.dim);
    c.lo.resize(c.dim);
    c.hi.resize(c.dim);
    c.coords.resize(c.dim);
    for (auto& p : c.periodic) std::scanf("%d", &p);
    for (auto& s : c.size) std::scanf("%lld", &s);
    for (int d = 0; d < c.dim; ++d) {
        char k[8];
        std::scanf("%7s", k);
        if (k[0] == 'U') {
            c.uniform[d] = 1;
            read_double(c.lo[d]);
            read_double(c.hi[d]);
        } else {
            long long n;
            std::scanf("%lld", &n);
            c.coords[d].resize(static_cast<size_t>(n));
            for (auto& v : c.coords[d]) read_double(v);
        }
    }
    long long n;
    std::scanf("%lld", &n);
    c.values.resize(static_cast<size_t>(n));
    for (auto& v : c.values) read_double(v);
    std::scanf("%lld", &n);
    c.points.resize(static_cast<size_t>(n) * c.dim);
    for (auto& v : c.points) read_double(v);
    std::scanf("%d", &c.nderiv);
    c.derivs.resize(static_cast<size_t>(c.nderiv) * c.dim);
    for (auto& v : c.derivs) std::scanf("%d", &v);
    return true;
}

struct Runner {
    virtual ~Runner() = default;
    virtual void run(const Case& c) = 0;
};

template <std::size_t D, std::size_t O>
struct FnRunner : Runner {
    intp::InterpolationFunction<double, D, O> f;
    explicit FnRunner(intp::InterpolationFunction<double, D, O>&& fn) : f(std::move(fn)) {}
    void run(const Case& c) override {
        const std::size_t np = c.points.size() / D;
        std::vector<double> single, batch(np * std::max(c.nderiv, 1));
        for (std::size_t p = 0; p < np; ++p) {
            std::array<double, D> x;
            for (std::size_t d = 0; d < D; ++d) x[d] = c.points[p * D + d];
            if (c.nderiv == 0) {
                single.push_back(f(x));
            } else {
                for (int k = 0; k < c.nderiv; ++k) {
                    std::array<std::size_t, D> kk;
                    for (std::size_t d = 0; d < D; ++d) kk[d] = static_cast<std::size_t>(c.derivs[k * D + d]);
                    single.push_back(f.derivative(x, kk));
                }
            }
        }
        f.evaluate(c.points.data(), np, batch.data(), c.nderiv ? c.derivs.data() : nullptr,
                   c.nderiv ? c.nderiv : 1);
        std::printf("%s %zu", c.name.c_str(), single.size());
        for (double v : single) std::printf(" %a", v);
        for (double v : batch) std::printf(" %a", v);
        std::printf("\n");
    }
};

template <std::size_t D, std::size_t O, typename... A>
std::unique_ptr<Runner> build(const Case& c, std::size_t axis, const intp::Mesh<double, D>& m, A... args) {
    if constexpr (sizeof...(A) == D) {
        std::array<bool, D> per{};
        for (std::size_t d = 0; d < D; ++d) per[d] = c.periodic[d] != 0;
        return std::unique_ptr<Runner>(new FnRunner<D, O>(intp::InterpolationFunction<double, D, O>(per, m, args...)));
    } else {
        if (c.uniform[axis])
            return build<D, O>(c, axis + 1, m, args..., std::make_pair(c.lo[axis], c.hi[axis]));
        const double* b = c.coords[axis].data();
        return build<D, O>(c, axis + 1, m, args..., std::make_pair(b, b + c.coords[axis].size()));
    }
}

template <std::size_t D, std::size_t O>
std::unique_ptr<Runner> make(const Case& c) {
    std::array<std::size_t, D> dims;
    for (std::size_t d = 0; d < D; ++d) dims[d] = static_cast<std::size_t>(c.size[d]);
    intp::Mesh<double, D> m{intp::MeshDimension<D>(dims)};
    for (std::size_t i = 0; i < m.size(); ++i) m(m.dimension().dimwise_indices(i)) = c.values[i];
    return build<D, O>(c, 0, m);
}

template <std::size_t D>
std::unique_ptr<Runner> make_d(const Case& c) {
    switch (c.order) {
        case 0: return make<D, 0>(c);
        case 1: return make<D, 1>(c);
        case 2: return make<D, 2>(c);
        case 3: return make<D, 3>(c);
        case 4: return make<D, 4>(c);
        case 5: return make<D, 5>(c);
        case 6: return make<D, 6>(c);
        case 7: return make<D, 7>(c);
    }
    return nullptr;
}

// Reference-shaped extras: range check, 1D forms, template reuse.
static int extras() {
    int bad = 0;
    intp::Mesh<double, 2> m(5, 5);
    for (std::size_t i = 0; i < 5; ++i)
        for (std::size_t j = 0; j < 5; ++j) m(i, j) = std::sin(0.3 * i) * std::cos(0.7 * j);
    intp::InterpolationFunction<double, 2, 3> f(m, std::make_pair(0., 4.), std::make_pair(0., 4.));
    try {
        f.at(-1, 1);
        std::printf("extra at() did not throw\n");
        ++bad;
    } catch (const std::domain_error&) {
    }
    try {
        f.derivative_at({-1.0, 1.0}, 1, 0);
        ++bad;
    } catch (const std::domain_error&) {
    }
    if (!(f.uniform(0) && f.uniform(1) && !f.periodicity(0) && f.get_order() == 3)) ++bad;
    if (f.range(1).second != 4.0 || f.spline().knots_num(0) != 9) ++bad;
    // template reuse: two meshes, one factorization
    intp::InterpolationFunctionTemplate<double, 2, 3> tpl({false, false}, intp::MeshDimension<2>(5, 5),
                                                          std::make_pair(0., 4.), std::make_pair(0., 4.));
    auto g1 = tpl.interpolate(m);
    intp::Mesh<double, 2> m2(5, 5);
    for (std::size_t i = 0; i < 25; ++i) m2(m2.dimension().dimwise_indices(i)) = 2.0 * m(m.dimension().dimwise_indices(i));
    auto g2 = tpl.interpolate(m2);
    const double a = g1(1.3, 2.2), b = g2(1.3, 2.2), c = f(1.3, 2.2);
    if (std::fabs(b - 2 * a) > 1e-13 || std::fabs(a - c) > 1e-15) {
        std::printf("extra template reuse mismatch %a %a %a\n", a, b, c);
        ++bad;
    }
    // 1D forms (Interpolation.hpp:509-540): range (0, n-1), periodic (0, n)
    std::vector<double> v{0.3, -0.1, 0.8, 0.5, -0.4, 0.2, 0.9};
    intp::InterpolationFunction1D<3> h(std::make_pair(v.begin(), v.end()));
    if (std::fabs(h(3.0) - v[3]) > 1e-14) ++bad;
    intp::InterpolationFunction1D<3> hp(std::make_pair(v.begin(), v.end()), true);
    if (std::fabs(hp(7.0) - v[0]) > 1e-14 || std::fabs(hp(2.0) - v[2]) > 1e-14) ++bad;
    intp::InterpolationFunctionTemplate1D<3> t1(v.size());
    auto h1 = t1.interpolate(std::make_pair(v.begin(), v.end()));
    if (std::fabs(h1(4.0) - v[4]) > 1e-14) ++bad;
    // vector-valued T (test/src/interpolation-test.cpp, interpolation on
    // vector): 31 points on the unit circle, periodic cubic of 2-vectors
    {
        constexpr std::size_t pn = 31;
        std::vector<std::array<float, 2>> pts;
        for (std::size_t i = 0; i < pn; ++i) {
            const double th = 2. * M_PI * static_cast<double>(i) / pn;
            pts.push_back({static_cast<float>(std::cos(th)), static_cast<float>(std::sin(th))});
        }
        intp::InterpolationFunction1D<3, std::array<float, 2>, float> circle(std::make_pair(pts.begin(), pts.end()),
                                                                              true);
        float err = 0;
        constexpr std::size_t sn = 1024;
        for (std::size_t i = 0; i < sn; ++i) {
            const float th = 2.f * static_cast<float>(M_PI) * static_cast<float>(i) / sn;
            const std::array<float, 2> p = circle(th);
            err += std::fabs(std::hypot(p[0], p[1]) - 1.f);
        }
        err /= sn;
        if (!(err < 1e-5f)) {
            std::printf("vector circle error %g\n", static_cast<double>(err));
            ++bad;
        }
        const auto cp = circle.spline().control_points();
        if (cp.size() != pn) ++bad;
    }
    // an allocation failure surfaces as the reference's std::bad_alloc
    // (aligned-allocator.hpp); intp_debug_fail_allocations injects one
    {
        intp_debug_fail_allocations(1);
        bool thrown = false;
        try {
            intp::InterpolationFunction1D<3> g(std::make_pair(v.begin(), v.end()));
            (void)g;
        } catch (const std::bad_alloc&) {
            thrown = true;
        }
        intp_debug_fail_allocations(0);
        if (!thrown) {
            std::printf("no bad_alloc on an allocation failure\n");
            ++bad;
        }
    }
    std::printf("extras %d\n", bad);
    return bad;
}

int main(int argc, char** argv) {
    if (argc > 1 && std::strcmp(argv[1], "extras") == 0) return extras();
    Case c;
    while (read_case(c)) {
        std::unique_ptr<Runner> r;
        try {
            switch (c.dim) {
                case 1: r = make_d<1>(c); break;
                case 2: r = make_d<2>(c); break;
                case 3: r = make_d<3>(c); break;
            }
            if (!r) {
                std::printf("%s unsupported\n", c.name.c_str());
                continue;
            }
            r->run(c);
        } catch (const std::exception& e) {
            std::printf("%s error %s\n", c.name.c_str(), e.what());
        }
        c = Case{};
    }
    return 0;
}
