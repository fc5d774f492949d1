/*
 * CPU oracle: plain-C restatement of the reference B-spline interpolation
 * algorithm (12ff54e/BSplineInterpolation). TEST INFRASTRUCTURE ONLY; see
 * intp_oracle.h for what it is used for and how it is pinned.
 *
 * Every function cites the reference file:line it follows. The arithmetic is
 * written in the same operation order as the reference so that, compiled with
 * -ffp-contract=off, results agree bit for bit with the reference headers.
 */
#define _POSIX_C_SOURCE 200809L
#include "intp_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static __thread char g_err[256];

static void set_err(const char* msg) {
    snprintf(g_err, sizeof g_err, "%s", msg);
}

const char* or_last_error(void) { return g_err; }

/* ------------------------------------------------------------------------ */
/* Band storage, BandMatrix.hpp:19-97 and ExtendedBandMatrix :99-181.        */
/* A(i,j) = B(j, i+q-j); right side band R(i, j+p-n) for j > i+q;            */
/* bottom side band S(j, i+q-n) for i > j+p.                                 */
/* ------------------------------------------------------------------------ */
typedef struct {
    int64_t n;
    int64_t p, q;
    int cyclic;
    double* bands;  /* n x (1+p+q) */
    double* right;  /* (n-q-1) x p */
    double* bottom; /* (n-p-1) x q */
} band_lu;

static double* main_ref(band_lu* m, int64_t i, int64_t j) {
    return &m->bands[j * (1 + m->p + m->q) + (i + m->q - j)];
}

static double* side_ref(band_lu* m, int64_t i, int64_t j) {
    /* ExtendedBandMatrix::side_bands_val, BandMatrix.hpp:122-128 */
    return j > i + m->q ? &m->right[i * m->p + (j + m->p - m->n)]
                        : &m->bottom[j * m->q + (i + m->q - m->n)];
}

static double* elem_ref(band_lu* m, int64_t i, int64_t j) {
    /* ExtendedBandMatrix::operator(), BandMatrix.hpp:138-146 */
    if (!m->cyclic) return main_ref(m, i, j);
    return (j > i + m->q || i > j + m->p) ? side_ref(m, i, j)
                                          : main_ref(m, i, j);
}

static int band_alloc(band_lu* m, int64_t n, int64_t p, int64_t q, int cyclic) {
    memset(m, 0, sizeof *m);
    m->n = n;
    m->p = p;
    m->q = q;
    m->cyclic = cyclic;
    m->bands = (double*)calloc((size_t)(n * (1 + p + q)), sizeof(double));
    if (!m->bands) return -1;
    if (cyclic) {
        int64_t nr = n - q - 1, nb = n - p - 1;
        if (nr < 0 || nb < 0) return -1;
        m->right = (double*)calloc((size_t)(nr * p + 1), sizeof(double));
        m->bottom = (double*)calloc((size_t)(nb * q + 1), sizeof(double));
        if (!m->right || !m->bottom) return -1;
    }
    return 0;
}

static void band_release(band_lu* m) {
    free(m->bands);
    free(m->right);
    free(m->bottom);
    memset(m, 0, sizeof *m);
}

static int64_t imin(int64_t a, int64_t b) { return a < b ? a : b; }
static int64_t imax(int64_t a, int64_t b) { return a > b ? a : b; }

/* BandLU<BandMatrix>::compute_impl, BandLU.hpp:103-118 */
static void band_factor(band_lu* m) {
    const int64_t n = m->n, p = m->p, q = m->q;
    for (int64_t k = 0; k + 1 < n; ++k) {
        for (int64_t i = k + 1; i < imin(k + p + 1, n); ++i)
            *main_ref(m, i, k) /= *main_ref(m, k, k);
        for (int64_t j = k + 1; j < imin(k + q + 1, n); ++j)
            for (int64_t i = k + 1; i < imin(k + p + 1, n); ++i)
                *main_ref(m, i, j) -= *main_ref(m, i, k) * *main_ref(m, k, j);
    }
}

/* BandLU<ExtendedBandMatrix>::compute_impl, BandLU.hpp:159-213 */
static void cyclic_factor(band_lu* m) {
    const int64_t n = m->n, p = m->p, q = m->q;
    for (int64_t k = 0; k + 1 < n; ++k) {
        for (int64_t i = k + 1; i < imin(k + p + 1, n); ++i)
            *main_ref(m, i, k) /= *main_ref(m, k, k);
        for (int64_t i = imax(n - q, k + p + 1); i < n; ++i)
            *side_ref(m, i, k) /= *main_ref(m, k, k);
        for (int64_t j = k + 1; j < imin(k + q + 1, n); ++j)
            for (int64_t i = k + 1; i < imin(k + p + 1, n); ++i)
                *main_ref(m, i, j) -= *main_ref(m, i, k) * *main_ref(m, k, j);
        for (int64_t i = k + 1; i < imin(k + p + 1, n); ++i)
            for (int64_t j = imax(n - p, k + q + 1); j < n; ++j)
                *elem_ref(m, i, j) -= *main_ref(m, i, k) * *side_ref(m, k, j);
        for (int64_t j = k + 1; j < imin(k + q + 1, n); ++j)
            for (int64_t i = imax(n - q, k + p + 1); i < n; ++i)
                *elem_ref(m, i, j) -= *side_ref(m, i, k) * *main_ref(m, k, j);
        if (k < imax(n - p - 1, n - q - 1)) {
            for (int64_t i = imax(n - q, k + p + 1); i < n; ++i)
                for (int64_t j = imax(n - p, k + q + 1); j < n; ++j)
                    *main_ref(m, i, j) -= *side_ref(m, i, k) * *side_ref(m, k, j);
        }
    }
}

/* BandLU<BandMatrix>::solve_in_place_impl, BandLU.hpp:120-143.
 * x is a strided line: element i at x[i*stride]. */
static void band_solve(band_lu* m, double* x, int64_t stride) {
    const int64_t n = m->n, p = m->p, q = m->q;
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = j + 1; i < imin(j + p + 1, n); ++i)
            x[i * stride] -= *main_ref(m, i, j) * x[j * stride];
    for (int64_t j = n - 1; j >= 0; --j) {
        x[j * stride] /= *main_ref(m, j, j);
        for (int64_t i = j < q ? 0 : j - q; i < j; ++i)
            x[i * stride] -= *main_ref(m, i, j) * x[j * stride];
    }
}

/* BandLU<ExtendedBandMatrix>::solve_in_place_impl, BandLU.hpp:215-259 */
static void cyclic_solve(band_lu* m, double* x, int64_t stride) {
    const int64_t n = m->n, p = m->p, q = m->q;
    for (int64_t j = 0; j < n; ++j) {
        for (int64_t i = j + 1; i < imin(j + p + 1, n); ++i)
            x[i * stride] -= *main_ref(m, i, j) * x[j * stride];
        if (j < n - p - 1)
            for (int64_t i = imax(n - q, j + p + 1); i < n; ++i)
                x[i * stride] -= *side_ref(m, i, j) * x[j * stride];
    }
    for (int64_t j = n - 1; j >= 0; --j) {
        x[j * stride] /= *main_ref(m, j, j);
        for (int64_t i = j < q ? 0 : j - q; i < j; ++i)
            x[i * stride] -= *main_ref(m, i, j) * x[j * stride];
        if (j > n - p - 1)
            for (int64_t i = 0; i < j - q; ++i)
                x[i * stride] -= *side_ref(m, i, j) * x[j * stride];
    }
}

/* ------------------------------------------------------------------------ */
/* Spline state                                                              */
/* ------------------------------------------------------------------------ */
struct or_spline {
    int dim, order;
    int periodic[OR_MAX_DIM];
    int uniform[OR_MAX_DIM];
    int64_t ncp[OR_MAX_DIM];     /* control points (= samples) per axis */
    double* knots[OR_MAX_DIM];
    int64_t nknots[OR_MAX_DIM];
    double lo[OR_MAX_DIM], hi[OR_MAX_DIM]; /* BSpline::range_ */
    double dx[OR_MAX_DIM];
    double* input_coords[OR_MAX_DIM];
    int64_t n_input[OR_MAX_DIM];
    band_lu solver[OR_MAX_DIM];
    int has_solver;
    double* ctrl;
    int64_t total;
};

/* BSpline::base_spline_value, BSpline.hpp:83-111. knots[seg] is the left
 * knot of the segment; out[] is right-aligned for spline_order < order. */
void or_base_spline_value(const double* knots, int64_t seg, double x,
                          int order, int spline_order, double* out) {
    for (int k = 0; k <= order; ++k) out[k] = 0.0;
    out[order] = 1.0;
    for (int i = 1; i <= spline_order; ++i) {
        const int idx_begin = order - i;
        for (int j = 0; j <= i; ++j) {
            const double* left = knots + seg - (i - j);
            const double* right = knots + seg + (j + 1);
            const double a = (j == 0) ? 0.0
                                      : out[idx_begin + j] * (x - *left) /
                                            (*(right - 1) - *left);
            const double b = (idx_begin + j == order)
                                 ? 0.0
                                 : out[idx_begin + j + 1] * (*right - x) /
                                       (*right - *(left + 1));
            out[idx_begin + j] = a + b;
        }
    }
}

/* std::upper_bound over [first, last) */
static int64_t upper_bound_idx(const double* a, int64_t first, int64_t last,
                               double x) {
    int64_t count = last - first;
    while (count > 0) {
        int64_t step = count / 2, it = first + step;
        if (!(x < a[it])) {
            first = it + 1;
            count -= step + 1;
        } else {
            count = step;
        }
    }
    return first;
}

/* BSpline::get_knot_iter, BSpline.hpp:125-157. Wraps x on periodic axes
 * (in place, as the reference does) and returns the knot-span index. */
static int64_t knot_iter(const or_spline* s, int d, double* x, int64_t hint,
                         int64_t last) {
    const double* t = s->knots[d];
    if (s->periodic[d]) {
        const double period = s->hi[d] - s->lo[d];
        *x = s->lo[d] + fmod(*x - s->lo[d], period) +
             (*x < s->lo[d] ? period : 0.0);
    }
    if (t[hint] <= *x && t[hint + 1] > *x) return hint;
    return upper_bound_idx(t, s->order + 1, last + 1, *x) - 1;
}

/* Hint of InterpolationFunction::add_hint_for_spline, Interpolation.hpp:277-295
 * (same expression in derivative_helper, :302-319). */
static int64_t knot_hint(const or_spline* s, int d, double c) {
    const int O = s->order;
    if (!s->uniform[d]) return O;
    double v = (c - s->lo[d]) / s->dx[d] -
               (s->periodic[d] ? 1.0 : 0.5 * (double)(O + 1));
    if (!(v > 0.0)) v = 0.0;
    v = ceil(v);
    const int64_t cap = s->nknots[d] - O - 2;
    /* the reference casts to size_t; clamp first so the cast is defined */
    if (v > (double)cap) return cap;
    int64_t h = (int64_t)v + O;
    return h < cap ? h : cap;
}

static int64_t locate(const or_spline* s, int d, double* x) {
    const int64_t h = knot_hint(s, d, *x);
    return knot_iter(s, d, x, h, s->nknots[d] - s->order - 2);
}

/* InterpolationFunction::create_knot_vector_ (uniform), Interpolation.hpp:322-362 */
static int knots_uniform(or_spline* s, int d, double x0, double x1) {
    const int O = s->order;
    const int per = s->periodic[d];
    const int64_t n = s->ncp[d] + (per ? 1 : 0);
    if (n < 2) {
        set_err("uniform axis needs at least 2 points");
        return -1;
    }
    s->uniform[d] = 1;
    s->dx[d] = (x1 - x0) / (double)(n - 1);
    const int64_t extra = per ? 2 * O + (1 - O % 2) : O + 1;
    const int64_t sz = n + extra;
    double* xs = (double*)malloc((size_t)sz * sizeof(double));
    if (!xs) {
        set_err("out of memory");
        return -1;
    }
    for (int64_t i = 0; i < sz; ++i) xs[i] = x0;
    if (per) {
        for (int64_t i = 0; i < sz; ++i)
            xs[i] = x0 + ((double)i - 0.5 * (double)extra) * s->dx[d];
    } else {
        for (int64_t i = O + 1; i < sz - O - 1; ++i)
            xs[i] = x0 + ((double)i - 0.5 * (double)extra) * s->dx[d];
        for (int64_t i = sz - O - 1; i < sz; ++i) xs[i] = x1;
    }
    s->knots[d] = xs;
    s->nknots[d] = sz;
    /* BSpline::load_knots, BSpline.hpp:222-227 */
    s->lo[d] = xs[O];
    s->hi[d] = xs[sz - O - (2 - O % 2)];
    return 0;
}

/* InterpolationFunction::create_knot_vector_ (non-uniform),
 * Interpolation.hpp:365-464 */
static int knots_nonuniform(or_spline* s, int d, const double* c) {
    const int O = s->order;
    const int per = s->periodic[d];
    const int64_t n = s->ncp[d] + (per ? 1 : 0);
    if (!per && O == 0) {
        /* the reference divides by the order here (:439) */
        set_err("non-uniform non-periodic axis needs order >= 1");
        return -1;
    }
    if (n < 2) {
        set_err("non-uniform axis needs at least 2 coordinates");
        return -1;
    }
    s->uniform[d] = 0;
    s->dx[d] = 0.0;
    const int64_t sz = per ? n + 2 * O + (1 - O % 2) : n + O + 1;
    double* xs = (double*)calloc((size_t)sz, sizeof(double));
    double* in = (double*)malloc((size_t)n * sizeof(double));
    if (!xs || !in) {
        free(xs);
        free(in);
        set_err("out of memory");
        return -1;
    }
    int64_t nin = 0;
    if (per) {
        int64_t it = 0;
        in[nin++] = c[it];
        for (int64_t i = O + 1; i < O + n; ++i) {
            const double present = c[++it];
            xs[i] = O % 2 == 0 ? 0.5 * (in[nin - 1] + present) : present;
            in[nin++] = present;
        }
        const double period = in[nin - 1] - in[0];
        for (int64_t i = 0; i < O + 1; ++i) {
            xs[i] = xs[n + i - 1] - period;
            xs[sz - i - 1] = xs[sz - i - n] + period;
        }
    } else {
        int64_t it = 0;
        const double l_knot = c[it];
        for (int64_t i = 0; i < O + 1; ++i) xs[i] = l_knot;
        in[nin++] = l_knot;
        double window_sum = 0.0;
        for (int64_t i = 1; i < O; ++i) {
            in[nin++] = c[++it];
            window_sum += in[i];
        }
        for (int64_t i = O + 1; i < n; ++i) {
            in[nin++] = c[++it];
            window_sum += in[i - 1];
            xs[i] = window_sum / (double)O;
            window_sum -= in[i - O];
        }
        const double r_knot = c[++it];
        for (int64_t i = n; i < n + O + 1; ++i) xs[i] = r_knot;
        in[nin++] = r_knot;
    }
    for (int64_t i = 0; i + 1 < nin; ++i) {
        if (!(in[i + 1] > in[i])) {
            free(xs);
            free(in);
            set_err("given coordinate is not monotonically increasing");
            return -1;
        }
    }
    s->knots[d] = xs;
    s->nknots[d] = sz;
    s->input_coords[d] = in;
    s->n_input[d] = nin;
    s->lo[d] = xs[O];
    s->hi[d] = xs[sz - O - (2 - O % 2)];
    return 0;
}

/* InterpolationFunctionTemplate::build_solver_, InterpolationTemplate.hpp:254-446
 * (C++17 branch: coefficients are placed with m(row, col)). */
static int build_solver(or_spline* s) {
    const int O = s->order;
    double base[64];
    for (int d = 0; d < s->dim; ++d) {
        const int per = s->periodic[d];
        const int uni = s->uniform[d];
        const int64_t n = s->ncp[d];
        const int64_t bw = per ? O / 2 : (O == 0 ? 0 : O - 1);
        band_lu* m = &s->solver[d];
        if (per && n < 2 * bw + 2) {
            set_err("periodic axis too short for this order");
            return -1;
        }
        if (band_alloc(m, n, bw, bw, per) != 0) {
            set_err("out of memory");
            return -1;
        }
        const double* t = s->knots[d];
        if (per && uni) {
            /* :273-280 */
            or_base_spline_value(t, O, t[O] + (double)(1 - O % 2) * s->dx[d] * 0.5,
                                 O, O, base);
        }
        for (int64_t i = 0; i < n; ++i) {
            if (!per && (i == 0 || i == n - 1)) {
                *elem_ref(m, i, i) = 1.0;
                continue;
            }
            const int64_t knot_num = s->nknots[d];
            int64_t knot_ind = 0;
            const int is_internal = i > O / 2 && i < n - O / 2 - 1;
            if (uni) {
                knot_ind = per ? i + O
                               : imin(knot_num - O - 2,
                                      i > O / 2 ? i + (O + 1) / 2 : O);
                if (!per) {
                    if (knot_ind <= 2 * O + 1 || knot_ind >= knot_num - 2 * O - 2) {
                        const double x = s->lo[d] + (double)i * s->dx[d];
                        or_base_spline_value(t, knot_ind, x, O, O, base);
                    }
                }
            } else {
                double x = s->input_coords[d][i];
                int64_t it;
                if (per) {
                    it = i + O;
                } else if (i == 0) {
                    it = O;
                } else if (i == s->n_input[d] - 1) {
                    it = knot_num - (O + 2);
                } else {
                    /* get_knot_iter on a non-periodic axis: no wrap */
                    const int64_t hint = i + 1;
                    const int64_t last = imin(knot_num - O - 1, i + O);
                    if (t[hint] <= x && t[hint + 1] > x)
                        it = hint;
                    else
                        it = upper_bound_idx(t, O + 1, last + 1, x) - 1;
                }
                knot_ind = it;
                or_base_spline_value(t, it, x, O, O, base);
            }
            const int64_t s_num = per ? (O | 1)
                                  : O == 1 ? 1
                                  : (uni && is_internal) ? (O | 1)
                                                         : O + 1;
            for (int64_t j = 0; j < s_num; ++j) {
                const int64_t row = (i + (per ? bw : 0)) % n;
                const int64_t col = (knot_ind - O + j) % n;
                *elem_ref(m, row, col) = base[j];
            }
        }
        if (per)
            cyclic_factor(m);
        else
            band_factor(m);
    }
    s->has_solver = 1;
    return 0;
}

or_spline* or_create(int dim, int order, const int* periodic,
                     const int64_t* sizes, const double* lo, const double* hi,
                     const double* const* coords) {
    if (dim < 1 || dim > OR_MAX_DIM || order < 0 || order > 63) {
        set_err("unsupported dimension or order");
        return NULL;
    }
    or_spline* s = (or_spline*)calloc(1, sizeof *s);
    if (!s) return NULL;
    s->dim = dim;
    s->order = order;
    s->total = 1;
    for (int d = 0; d < dim; ++d) {
        s->periodic[d] = periodic ? (periodic[d] != 0) : 0;
        s->ncp[d] = sizes[d];
        if (sizes[d] < 1) {
            set_err("empty axis");
            or_free(s);
            return NULL;
        }
        s->total *= sizes[d];
    }
    for (int d = 0; d < dim; ++d) {
        int rc = (coords && coords[d]) ? knots_nonuniform(s, d, coords[d])
                                       : knots_uniform(s, d, lo[d], hi[d]);
        if (rc != 0) {
            or_free(s);
            return NULL;
        }
    }
    if (build_solver(s) != 0) {
        or_free(s);
        return NULL;
    }
    s->ctrl = (double*)calloc((size_t)s->total, sizeof(double));
    if (!s->ctrl) {
        or_free(s);
        return NULL;
    }
    return s;
}

or_spline* or_create_from_knots(int dim, int order, const int* periodic,
                                const int64_t* ncp, const double* const* knots,
                                const int64_t* nknots, const double* ctrl) {
    if (dim < 1 || dim > OR_MAX_DIM || order < 0 || order > 63) {
        set_err("unsupported dimension or order");
        return NULL;
    }
    or_spline* s = (or_spline*)calloc(1, sizeof *s);
    if (!s) return NULL;
    s->dim = dim;
    s->order = order;
    s->total = 1;
    for (int d = 0; d < dim; ++d) {
        s->periodic[d] = periodic ? (periodic[d] != 0) : 0;
        s->ncp[d] = ncp[d];
        s->total *= ncp[d];
        s->uniform[d] = 0; /* BSpline::operator()(DimArray<double>) uses hint O */
        s->nknots[d] = nknots[d];
        s->knots[d] = (double*)malloc((size_t)nknots[d] * sizeof(double));
        memcpy(s->knots[d], knots[d], (size_t)nknots[d] * sizeof(double));
        /* BSpline constructor, BSpline.hpp:200-202 */
        s->lo[d] = knots[d][order];
        s->hi[d] = knots[d][nknots[d] - order - 1];
    }
    s->ctrl = (double*)malloc((size_t)s->total * sizeof(double));
    memcpy(s->ctrl, ctrl, (size_t)s->total * sizeof(double));
    return s;
}

void or_free(or_spline* s) {
    if (!s) return;
    for (int d = 0; d < OR_MAX_DIM; ++d) {
        free(s->knots[d]);
        free(s->input_coords[d]);
        band_release(&s->solver[d]);
    }
    free(s->ctrl);
    free(s);
}

/* ------------------------------------------------------------------------ */
/* Control-point solve, InterpolationTemplate.hpp:448-580                    */
/* ------------------------------------------------------------------------ */
typedef struct {
    or_spline* s;
    int axis;
    int64_t begin, end; /* line range */
    int64_t n, stride;  /* line length and element stride */
} solve_task;

static void* solve_lines(void* arg) {
    solve_task* tk = (solve_task*)arg;
    or_spline* s = tk->s;
    band_lu* m = &s->solver[tk->axis];
    const int64_t n = tk->n, stride = tk->stride;
    for (int64_t l = tk->begin; l < tk->end; ++l) {
        /* line l = (outer o, inner t): start o*n*stride + t */
        const int64_t o = l / stride, t = l % stride;
        double* x = s->ctrl + o * n * stride + t;
        if (m->cyclic)
            cyclic_solve(m, x, stride);
        else
            band_solve(m, x, stride);
    }
    return NULL;
}

int or_interpolate(or_spline* s, const double* values, int nthreads) {
    if (!s->has_solver) {
        set_err("spline has no solver");
        return -1;
    }
    const int D = s->dim, O = s->order;
    /* periodic shift of O/2 on load, :451-462 */
    int64_t idx[OR_MAX_DIM];
    for (int64_t lin = 0; lin < s->total; ++lin) {
        int64_t r = lin;
        for (int d = D - 1; d >= 0; --d) {
            idx[d] = r % s->ncp[d];
            r /= s->ncp[d];
        }
        int64_t dst = 0;
        for (int d = 0; d < D; ++d) {
            int64_t i = idx[d];
            if (s->periodic[d]) i = (i + s->ncp[d] + O / 2) % s->ncp[d];
            dst = dst * s->ncp[d] + i;
        }
        s->ctrl[dst] = values[lin];
    }
    /* D passes: the reference solves the last axis of a tensor that it rotates
     * after each pass (:502-573), i.e. axis D-1 first, then D-2, ..., 0. The
     * rotation only moves data, so lines are solved in place here. */
    if (nthreads < 1) nthreads = 1;
    for (int pass = 0; pass < D; ++pass) {
        const int axis = D - 1 - pass;
        int64_t stride = 1;
        for (int d = axis + 1; d < D; ++d) stride *= s->ncp[d];
        const int64_t n = s->ncp[axis];
        const int64_t lines = s->total / n;
        int nt = nthreads;
        if (nt > lines) nt = (int)lines;
        pthread_t th[256];
        solve_task tk[256];
        if (nt > 256) nt = 256;
        for (int k = 0; k < nt; ++k) {
            tk[k].s = s;
            tk[k].axis = axis;
            tk[k].begin = lines * k / nt;
            tk[k].end = lines * (k + 1) / nt;
            tk[k].n = n;
            tk[k].stride = stride;
        }
        if (nt == 1) {
            solve_lines(&tk[0]);
        } else {
            for (int k = 0; k < nt; ++k) pthread_create(&th[k], NULL, solve_lines, &tk[k]);
            for (int k = 0; k < nt; ++k) pthread_join(th[k], NULL);
        }
    }
    return 0;
}

int or_set_control_points(or_spline* s, const double* ctrl) {
    memcpy(s->ctrl, ctrl, (size_t)s->total * sizeof(double));
    return 0;
}

int or_get_control_points(const or_spline* s, double* out) {
    memcpy(out, s->ctrl, (size_t)s->total * sizeof(double));
    return 0;
}

int64_t or_num_knots(const or_spline* s, int axis) { return s->nknots[axis]; }
int64_t or_num_ctrl(const or_spline* s, int axis) { return s->ncp[axis]; }

int or_get_knots(const or_spline* s, int axis, double* out) {
    memcpy(out, s->knots[axis], (size_t)s->nknots[axis] * sizeof(double));
    return 0;
}

int or_get_range(const or_spline* s, int axis, double* lo, double* hi) {
    *lo = s->lo[axis];
    *hi = s->hi[axis];
    return 0;
}

double or_get_dx(const or_spline* s, int axis) { return s->dx[axis]; }
int or_is_uniform(const or_spline* s, int axis) { return s->uniform[axis]; }

/* ------------------------------------------------------------------------ */
/* Evaluation                                                                */
/* ------------------------------------------------------------------------ */

static int64_t ipow(int64_t b, int e) {
    int64_t r = 1;
    while (e-- > 0) r *= b;
    return r;
}

/* BSpline::operator(), BSpline.hpp:305-335 with the INTP_CELL_LAYOUT
 * contraction: local index digit d = (i / (O+1)^d) % (O+1), coefficient
 * cp * b0 * b1 * ..., summed in increasing i. */
static double eval_value(const or_spline* s, const double* c) {
    const int D = s->dim, O = s->order, W = O + 1;
    double x[OR_MAX_DIM];
    int64_t cell[OR_MAX_DIM];
    double base[OR_MAX_DIM][64];
    for (int d = 0; d < D; ++d) {
        x[d] = c[d];
        cell[d] = locate(s, d, &x[d]);
        or_base_spline_value(s->knots[d], cell[d], x[d], O, O, base[d]);
    }
    const int64_t buf = ipow(W, D);
    double v = 0.0;
    for (int64_t i = 0; i < buf; ++i) {
        int64_t lin = 0, comb = i;
        int dig[OR_MAX_DIM];
        for (int d = 0; d < D; ++d) {
            dig[d] = (int)(comb % W);
            comb /= W;
        }
        for (int d = 0; d < D; ++d) {
            int64_t k = cell[d] - O + dig[d];
            if (s->periodic[d]) k %= s->ncp[d];
            lin = lin * s->ncp[d] + k;
        }
        double coef = s->ctrl[lin];
        for (int d = 0; d < D; ++d) coef *= base[d][dig[d]];
        v += coef;
    }
    return v;
}

/* BSpline::derivative_at, BSpline.hpp:393-532 */
static double eval_deriv(const or_spline* s, const double* c, const int* k) {
    const int D = s->dim, O = s->order, W = O + 1;
    int sorder[OR_MAX_DIM];
    for (int d = 0; d < D; ++d) {
        sorder[d] = O >= k[d] ? O - k[d] : O + 1;
        if (sorder[d] > O) return 0.0;
    }
    double x[OR_MAX_DIM];
    int64_t cell[OR_MAX_DIM];
    double base[OR_MAX_DIM][64];
    for (int d = 0; d < D; ++d) {
        x[d] = c[d];
        cell[d] = locate(s, d, &x[d]);
        or_base_spline_value(s->knots[d], cell[d], x[d], O, sorder[d], base[d]);
    }
    const int64_t buf = ipow(W, D);
    double lcp[4096], lsv[4096];
    if (buf > 4096) return NAN;
    /* local meshes are row-major over (O+1)^D, last index fastest */
    for (int64_t i = 0; i < buf; ++i) {
        int dig[OR_MAX_DIM];
        int64_t comb = i;
        for (int d = 0; d < D; ++d) {
            dig[d] = (int)(comb % W);
            comb /= W;
        }
        double coef = 1.0;
        int64_t lin = 0, loc = 0;
        for (int d = 0; d < D; ++d) {
            coef *= base[d][dig[d]];
            int64_t kk = dig[d] + (cell[d] - O);
            if (s->periodic[d]) kk %= s->ncp[d];
            lin = lin * s->ncp[d] + kk;
            loc = loc * W + dig[d];
        }
        lsv[loc] = coef;
        lcp[loc] = s->ctrl[lin];
    }
    for (int d = 0; d < D; ++d) {
        if (sorder[d] == O) continue;
        const int64_t hs = buf / W;
        const int64_t dstride = ipow(W, D - 1 - d);
        const double* t = s->knots[d];
        for (int64_t i = 0; i < hs; ++i) {
            int lidx[OR_MAX_DIM] = {0, 0, 0, 0};
            int64_t comb = i;
            for (int dd = 0; dd < D; ++dd) {
                if (dd == d) continue;
                lidx[dd] = (int)(comb % W);
                comb /= W;
            }
            int64_t start = 0;
            for (int dd = 0; dd < D; ++dd) start = start * W + (dd == d ? 0 : lidx[dd]);
            double* it = lcp + start;
            for (int kk = O; kk > sorder[d]; --kk) {
                for (int j = kk; j > 0; --j) {
                    const int64_t a = O + j - kk;
                    it[a * dstride] = (double)kk * (it[a * dstride] - it[(a - 1) * dstride]) /
                                      (t[cell[d] + j] - t[cell[d] + j - kk]);
                }
            }
        }
    }
    double v = 0.0;
    for (int64_t i = 0; i < buf; ++i) v += lsv[i] * lcp[i];
    return v;
}

/* The same two functions with the dimension and order as compile-time
 * constants (the reference is templated on both, which lets the compiler
 * unroll and register-allocate the local arrays); arithmetic unchanged. */
#define OR_DEFINE_EVAL(SUF, DIM_, ORD_) \
static double eval_value_##SUF(const or_spline* s, const double* c) { \
    const int D = DIM_, O = ORD_, W = ORD_ + 1; \
    double x[OR_MAX_DIM]; \
    int64_t cell[OR_MAX_DIM]; \
    double base[OR_MAX_DIM][64]; \
    for (int d = 0; d < D; ++d) { \
        x[d] = c[d]; \
        cell[d] = locate(s, d, &x[d]); \
        or_base_spline_value(s->knots[d], cell[d], x[d], O, O, base[d]); \
    } \
    const int64_t buf = ipow(W, D); \
    double v = 0.0; \
    for (int64_t i = 0; i < buf; ++i) { \
        int64_t lin = 0, comb = i; \
        int dig[OR_MAX_DIM]; \
        for (int d = 0; d < D; ++d) { \
            dig[d] = (int)(comb % W); \
            comb /= W; \
        } \
        for (int d = 0; d < D; ++d) { \
            int64_t k = cell[d] - O + dig[d]; \
            if (s->periodic[d]) k %= s->ncp[d]; \
            lin = lin * s->ncp[d] + k; \
        } \
        double coef = s->ctrl[lin]; \
        for (int d = 0; d < D; ++d) coef *= base[d][dig[d]]; \
        v += coef; \
    } \
    return v; \
} \
 \
static double eval_deriv_##SUF(const or_spline* s, const double* c, const int* k) { \
    const int D = DIM_, O = ORD_, W = ORD_ + 1; \
    int sorder[OR_MAX_DIM]; \
    for (int d = 0; d < D; ++d) { \
        sorder[d] = O >= k[d] ? O - k[d] : O + 1; \
        if (sorder[d] > O) return 0.0; \
    } \
    double x[OR_MAX_DIM]; \
    int64_t cell[OR_MAX_DIM]; \
    double base[OR_MAX_DIM][64]; \
    for (int d = 0; d < D; ++d) { \
        x[d] = c[d]; \
        cell[d] = locate(s, d, &x[d]); \
        or_base_spline_value(s->knots[d], cell[d], x[d], O, sorder[d], base[d]); \
    } \
    const int64_t buf = ipow(W, D); \
    double lcp[4096], lsv[4096]; \
    if (buf > 4096) return NAN; \
    for (int64_t i = 0; i < buf; ++i) { \
        int dig[OR_MAX_DIM]; \
        int64_t comb = i; \
        for (int d = 0; d < D; ++d) { \
            dig[d] = (int)(comb % W); \
            comb /= W; \
        } \
        double coef = 1.0; \
        int64_t lin = 0, loc = 0; \
        for (int d = 0; d < D; ++d) { \
            coef *= base[d][dig[d]]; \
            int64_t kk = dig[d] + (cell[d] - O); \
            if (s->periodic[d]) kk %= s->ncp[d]; \
            lin = lin * s->ncp[d] + kk; \
            loc = loc * W + dig[d]; \
        } \
        lsv[loc] = coef; \
        lcp[loc] = s->ctrl[lin]; \
    } \
    for (int d = 0; d < D; ++d) { \
        if (sorder[d] == O) continue; \
        const int64_t hs = buf / W; \
        const int64_t dstride = ipow(W, D - 1 - d); \
        const double* t = s->knots[d]; \
        for (int64_t i = 0; i < hs; ++i) { \
            int lidx[OR_MAX_DIM] = {0, 0, 0, 0}; \
            int64_t comb = i; \
            for (int dd = 0; dd < D; ++dd) { \
                if (dd == d) continue; \
                lidx[dd] = (int)(comb % W); \
                comb /= W; \
            } \
            int64_t start = 0; \
            for (int dd = 0; dd < D; ++dd) start = start * W + (dd == d ? 0 : lidx[dd]); \
            double* it = lcp + start; \
            for (int kk = O; kk > sorder[d]; --kk) { \
                for (int j = kk; j > 0; --j) { \
                    const int64_t a = O + j - kk; \
                    it[a * dstride] = (double)kk * (it[a * dstride] - it[(a - 1) * dstride]) / \
                                      (t[cell[d] + j] - t[cell[d] + j - kk]); \
                } \
            } \
        } \
    } \
    double v = 0.0; \
    for (int64_t i = 0; i < buf; ++i) v += lsv[i] * lcp[i]; \
    return v; \
} \

OR_DEFINE_EVAL(1_0, 1, 0)
OR_DEFINE_EVAL(1_1, 1, 1)
OR_DEFINE_EVAL(1_2, 1, 2)
OR_DEFINE_EVAL(1_3, 1, 3)
OR_DEFINE_EVAL(1_4, 1, 4)
OR_DEFINE_EVAL(1_5, 1, 5)
OR_DEFINE_EVAL(1_6, 1, 6)
OR_DEFINE_EVAL(1_7, 1, 7)
OR_DEFINE_EVAL(2_0, 2, 0)
OR_DEFINE_EVAL(2_1, 2, 1)
OR_DEFINE_EVAL(2_2, 2, 2)
OR_DEFINE_EVAL(2_3, 2, 3)
OR_DEFINE_EVAL(2_4, 2, 4)
OR_DEFINE_EVAL(2_5, 2, 5)
OR_DEFINE_EVAL(2_6, 2, 6)
OR_DEFINE_EVAL(2_7, 2, 7)
OR_DEFINE_EVAL(3_0, 3, 0)
OR_DEFINE_EVAL(3_1, 3, 1)
OR_DEFINE_EVAL(3_2, 3, 2)
OR_DEFINE_EVAL(3_3, 3, 3)
OR_DEFINE_EVAL(3_4, 3, 4)
OR_DEFINE_EVAL(3_5, 3, 5)
OR_DEFINE_EVAL(3_6, 3, 6)
OR_DEFINE_EVAL(3_7, 3, 7)

typedef double (*or_value_fn)(const or_spline*, const double*);
typedef double (*or_deriv_fn)(const or_spline*, const double*, const int*);
static const or_value_fn k_value_fns[3][8] = {
    {eval_value_1_0, eval_value_1_1, eval_value_1_2, eval_value_1_3, eval_value_1_4, eval_value_1_5, eval_value_1_6, eval_value_1_7},
    {eval_value_2_0, eval_value_2_1, eval_value_2_2, eval_value_2_3, eval_value_2_4, eval_value_2_5, eval_value_2_6, eval_value_2_7},
    {eval_value_3_0, eval_value_3_1, eval_value_3_2, eval_value_3_3, eval_value_3_4, eval_value_3_5, eval_value_3_6, eval_value_3_7}};
static const or_deriv_fn k_deriv_fns[3][8] = {
    {eval_deriv_1_0, eval_deriv_1_1, eval_deriv_1_2, eval_deriv_1_3, eval_deriv_1_4, eval_deriv_1_5, eval_deriv_1_6, eval_deriv_1_7},
    {eval_deriv_2_0, eval_deriv_2_1, eval_deriv_2_2, eval_deriv_2_3, eval_deriv_2_4, eval_deriv_2_5, eval_deriv_2_6, eval_deriv_2_7},
    {eval_deriv_3_0, eval_deriv_3_1, eval_deriv_3_2, eval_deriv_3_3, eval_deriv_3_4, eval_deriv_3_5, eval_deriv_3_6, eval_deriv_3_7}};

typedef struct {
    const or_spline* s;
    const double* coords;
    const int* derivs;
    int nderiv;
    double* out;
    int64_t begin, end;
} eval_task;

static void* eval_points(void* arg) {
    eval_task* tk = (eval_task*)arg;
    const int D = tk->s->dim, O = tk->s->order;
    const int spec = D >= 1 && D <= 3 && O <= 7;
    const or_value_fn vf = spec ? k_value_fns[D - 1][O] : eval_value;
    const or_deriv_fn df = spec ? k_deriv_fns[D - 1][O] : eval_deriv;
    for (int64_t p = tk->begin; p < tk->end; ++p) {
        const double* c = tk->coords + p * D;
        if (!tk->derivs) {
            tk->out[p] = vf(tk->s, c);
        } else {
            for (int r = 0; r < tk->nderiv; ++r)
                tk->out[p * tk->nderiv + r] = df(tk->s, c, tk->derivs + r * D);
        }
    }
    return NULL;
}

static int run_eval(const or_spline* s, const double* coords, int64_t npts,
                    const int* derivs, int nderiv, double* out, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if (npts < 1024) nthreads = 1;
    pthread_t th[256];
    eval_task tk[256];
    for (int k = 0; k < nthreads; ++k) {
        tk[k].s = s;
        tk[k].coords = coords;
        tk[k].derivs = derivs;
        tk[k].nderiv = nderiv;
        tk[k].out = out;
        tk[k].begin = npts * k / nthreads;
        tk[k].end = npts * (k + 1) / nthreads;
    }
    if (nthreads == 1) {
        eval_points(&tk[0]);
        return 0;
    }
    for (int k = 0; k < nthreads; ++k) pthread_create(&th[k], NULL, eval_points, &tk[k]);
    for (int k = 0; k < nthreads; ++k) pthread_join(th[k], NULL);
    return 0;
}

int or_eval(const or_spline* s, const double* coords, int64_t npts,
            double* out, int nthreads) {
    return run_eval(s, coords, npts, NULL, 0, out, nthreads);
}

int or_eval_deriv(const or_spline* s, const double* coords, int64_t npts,
                  const int* derivs, int nderiv, double* out, int nthreads) {
    return run_eval(s, coords, npts, derivs, nderiv, out, nthreads);
}

int or_locate(const or_spline* s, const double* coords, int64_t npts,
              int64_t* cells, double* wrapped) {
    const int D = s->dim;
    for (int64_t p = 0; p < npts; ++p) {
        for (int d = 0; d < D; ++d) {
            double x = coords[p * D + d];
            cells[p * D + d] = locate(s, d, &x);
            if (wrapped) wrapped[p * D + d] = x;
        }
    }
    return 0;
}

int or_in_range(const or_spline* s, const double* coord) {
    for (int d = 0; d < s->dim; ++d)
        if (!s->periodic[d] && (coord[d] < s->lo[d] || coord[d] > s->hi[d])) return 0;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* Standalone band solve for the band-matrix tests                           */
/* (test/src/band-matrix-and-solver-test.cpp)                                */
/* ------------------------------------------------------------------------ */
int or_band_solve_dense(int64_t n, int p, int q, int cyclic, const double* a,
                        double* b) {
    band_lu m;
    if (band_alloc(&m, n, p, q, cyclic) != 0) {
        band_release(&m);
        set_err("bad band shape");
        return -1;
    }
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t j = 0; j < n; ++j) {
            const int in_main = (j + p >= i) && (i + q >= j);
            int in_side = 0;
            if (cyclic)
                in_side = (j >= imax(n - p, i + q + 1)) || (i >= imax(n - q, j + p + 1));
            if (in_main || in_side) *elem_ref(&m, i, j) = a[i * n + j];
        }
    }
    if (cyclic) {
        cyclic_factor(&m);
        cyclic_solve(&m, b, 1);
    } else {
        band_factor(&m);
        band_solve(&m, b, 1);
    }
    band_release(&m);
    return 0;
}
