// Host-side check of the table model (knots, collocation, factors) without a
// GPU. Reads cases from stdin:
//   dim order  periodic[dim] size[dim]  lo[dim] hi[dim]  ncoords[dim] coords...
// and prints, per case: the knots of every axis and the max residual of
// L*U against the collocation matrix and of A*(LU \ b) against b.
// Built with -fsanitize=address by tests/test_host_model.py.
#include <cmath>
#include <cstdio>
#include <vector>

#include "spline_model.hpp"

using namespace intp_gb300;

static double lu_solve_residual(const AxisModel& ax) {
    const int64_t n = ax.n;
    std::vector<double> b(n), x(n), y(n);
    for (int64_t i = 0; i < n; ++i) b[i] = std::sin(1.0 + 0.37 * static_cast<double>(i));
    // solve with the GPU row layout of the factor, as the kernels do
    const LineFactor& f = ax.factor;
    const int64_t p = f.p, q = f.q;
    x = b;
    std::vector<double> acc(q > 0 ? q : 1);
    for (int64_t r = 0; r < q; ++r) acc[r] = f.cyclic ? x[n - q + r] : 0.0;
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
    // y = A x through the stencil
    double err = 0.0, nb = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        double s = 0.0;
        for (int w = 0; w < ax.stencil.width; ++w)
            s += ax.stencil.val[i * ax.stencil.width + w] * x[ax.stencil.col[i * ax.stencil.width + w]];
        err = std::fmax(err, std::fabs(s - b[i]));
        nb = std::fmax(nb, std::fabs(b[i]));
    }
    // and through BandStore::multiply
    ax.colloc.multiply(x.data(), y.data());
    for (int64_t i = 0; i < n; ++i) err = std::fmax(err, std::fabs(y[i] - b[i]));
    return err / nb;
}

int main() {
    int dim, order;
    while (std::scanf("%d %d", &dim, &order) == 2) {
        TableSpec spec;
        spec.dim = dim;
        spec.order = order;
        std::vector<std::vector<double>> coords(dim);
        for (int d = 0; d < dim; ++d) {
            int p;
            if (std::scanf("%d", &p) != 1) return 2;
            spec.periodic[d] = p != 0;
        }
        for (int d = 0; d < dim; ++d) {
            long long s;
            if (std::scanf("%lld", &s) != 1) return 2;
            spec.size[d] = s;
        }
        for (int d = 0; d < dim; ++d)
            if (std::scanf("%la", &spec.lo[d]) != 1) return 2;
        for (int d = 0; d < dim; ++d)
            if (std::scanf("%la", &spec.hi[d]) != 1) return 2;
        for (int d = 0; d < dim; ++d) {
            long long nc;
            if (std::scanf("%lld", &nc) != 1) return 2;
            coords[d].resize(static_cast<size_t>(nc));
            for (long long i = 0; i < nc; ++i)
                if (std::scanf("%la", &coords[d][i]) != 1) return 2;
            spec.coords[d] = nc ? coords[d].data() : nullptr;
        }
        TableModel m;
        const std::string err = build_model(spec, m);
        if (!err.empty()) {
            std::printf("ERROR %s\n", err.c_str());
            continue;
        }
        std::printf("OK\n");
        for (int d = 0; d < dim; ++d) {
            const AxisModel& ax = m.axis[d];
            std::printf("K %zu", ax.knots.size());
            for (double v : ax.knots) std::printf(" %a", v);
            std::printf("\nR %a %a %.3e\n", ax.range_lo, ax.range_hi, lu_solve_residual(ax));
        }
    }
    return 0;
}
