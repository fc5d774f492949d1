/*
 * CPU oracle for the B-spline control-point solve and evaluation.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference
 * library's algorithm (12ff54e/BSplineInterpolation, header-only C++ under
 * src/include/), used as the checker by the test suite, by the smoke entry and
 * by the CPU-baseline leg of the benchmark. The product (the CUDA library under
 * bsplineinterpolation_gb300/) never links, loads or calls it.
 *
 * Semantics follow the reference's test build: INTP_PERIODIC_NO_DUMMY_POINT
 * defined (test/CMakeLists.txt:46-47), so a periodic axis of n samples has n
 * control points and the period is given by the axis range. Value evaluation
 * follows the INTP_CELL_LAYOUT contraction order (BSpline.hpp:320-335), read
 * from the plain control-point array (the cell layout only duplicates values).
 *
 * The oracle is compiled with -ffp-contract=off so that it rounds exactly like
 * the reference built for x86-64 (no fused multiply-add) on every host.
 *
 * Parity pin: tests/test_oracle_golden.py checks it against the golden vectors
 * of the reference's own tests (test/src/interpolation-test.cpp,
 * test/src/bspline-test.cpp, test/src/band-matrix-and-solver-test.cpp), and
 * tests/test_oracle_vs_ref.py checks it bit-for-bit against the reference
 * headers compiled by oracle/build_ref.sh where those headers are present.
 */
#ifndef INTP_ORACLE_H
#define INTP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_MAX_DIM 4

typedef struct or_spline or_spline;

/* Build knots, collocation matrices and their band LU factors.
 * sizes[d]: samples along axis d (NO_DUMMY: a periodic axis holds one period
 * without the repeated end point). coords[d] == NULL: uniform axis on
 * [lo[d], hi[d]]; else coords[d] holds sizes[d] (+1 if periodic) increasing
 * sample coordinates and lo/hi are ignored.
 * Returns NULL on error; or_last_error() tells why. */
or_spline* or_create(int dim, int order, const int* periodic,
                     const int64_t* sizes, const double* lo, const double* hi,
                     const double* const* coords);
void or_free(or_spline* s);
const char* or_last_error(void);

/* Solve for control points from a row-major value mesh (sizes[] as given). */
int or_interpolate(or_spline* s, const double* values, int nthreads);
/* Load control points directly (row-major, same shape as the value mesh). */
int or_set_control_points(or_spline* s, const double* ctrl);
/* Copy control points out (row-major). */
int or_get_control_points(const or_spline* s, double* out);

int64_t or_num_knots(const or_spline* s, int axis);
int or_get_knots(const or_spline* s, int axis, double* out);
int or_get_range(const or_spline* s, int axis, double* lo, double* hi);
double or_get_dx(const or_spline* s, int axis);
int or_is_uniform(const or_spline* s, int axis);
int64_t or_num_ctrl(const or_spline* s, int axis);

/* Value at npts points (coords row-major npts x dim), operator() semantics. */
int or_eval(const or_spline* s, const double* coords, int64_t npts,
            double* out, int nthreads);
/* Derivatives: nderiv rows of dim orders; out is npts x nderiv.
 * derivative() semantics (no range check). */
int or_eval_deriv(const or_spline* s, const double* coords, int64_t npts,
                  const int* derivs, int nderiv, double* out, int nthreads);
/* Knot-span index per axis (npts x dim) and the periodic-wrapped coordinate. */
int or_locate(const or_spline* s, const double* coords, int64_t npts,
              int64_t* cells, double* wrapped);
/* 1 if every non-periodic coordinate lies in its axis range, else 0
 * (Interpolation.hpp:482-491). */
int or_in_range(const or_spline* s, const double* coord);

/* Spline from explicit knots and control points (BSpline.hpp:188-210).
 * knots[d] has nknots[d] entries; ctrl is row-major with ncp[d] per axis. */
or_spline* or_create_from_knots(int dim, int order, const int* periodic,
                                const int64_t* ncp, const double* const* knots,
                                const int64_t* nknots, const double* ctrl);

/* Standalone band LU (BandLU.hpp). Dense input a (n x n row-major, only the
 * band and, for cyclic, the side bands are read). Solves in place for b. */
int or_band_solve_dense(int64_t n, int p, int q, int cyclic, const double* a,
                        double* b);

/* Basis values (BSpline.hpp:83-111): out[0..order]. */
void or_base_spline_value(const double* knots, int64_t seg, double x,
                          int order, int spline_order, double* out);

#ifdef __cplusplus
}
#endif

#endif
