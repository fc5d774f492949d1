// Core of the MATLAB binding (bspline_gpu.cpp): the reference MEX function's
// argument conventions (matlab/bspline.cpp:63-141 of the reference) mapped
// onto this library's C-ABI, with no MATLAB types, so it can be built and
// tested without MATLAB.
//
// Arguments, as the reference's bspline(order, is_periodic, range, mesh,
// coords, derivative) receives them:
//   order       spline order
//   dim         number of mesh dimensions larger than 1
//   periodic    dim flags, one per MATLAB dimension
//   range       dim x 2 doubles, column-major: range(j, 0) = x_min and
//               range(j, 1) = x_max of MATLAB dimension j
//   mesh        the value array, column-major, MATLAB dimensions dims[0..dim)
//   coords      npts x dim doubles, column-major: point i, MATLAB dimension j
//               at coords[i + j * npts]
//   derivative  dim derivative orders, one per MATLAB dimension
//   result      npts doubles
// The reference binds MATLAB dimension j to axis dim-1-j of its C++
// interpolant, so the column-major mesh is the row-major mesh of reversed
// dimensions, unchanged in memory. Periodic axes here take n samples as n
// control points (the reference MEX appended an unused dummy point for the
// same effect). Returns an empty string on success, else the reason.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "intp_gpu.h"

namespace intp_matlab {

inline std::string bspline_eval(uint64_t order, int dim, const bool* periodic, const double* range,
                                const double* mesh, const size_t* dims, const double* coords, size_t npts,
                                const uint64_t* derivative, double* result) {
    if (dim < 1 || dim > INTP_GPU_MAX_DIM) return "unsupported dimension " + std::to_string(dim);
    if (order > INTP_GPU_MAX_ORDER) return "unsupported order " + std::to_string(order);
    intp_table_desc desc{};
    desc.dim = dim;
    desc.order = static_cast<int32_t>(order);
    desc.precision = INTP_PRECISION_FP64;
    desc.refine_steps = 0;
    desc.channels = 1;
    std::vector<int32_t> deriv(static_cast<size_t>(dim));
    for (int k = 0; k < dim; ++k) {
        const int j = dim - 1 - k;  // MATLAB dimension of axis k
        desc.periodic[k] = periodic[j] ? 1 : 0;
        desc.size[k] = static_cast<int64_t>(dims[j]);
        desc.range_lo[k] = range[j];
        desc.range_hi[k] = range[j + dim];
        deriv[static_cast<size_t>(k)] = static_cast<int32_t>(derivative[j]);
    }
    // row-major points with the axes in C++ order
    std::vector<double> pts(npts * static_cast<size_t>(dim));
    for (size_t i = 0; i < npts; ++i)
        for (int k = 0; k < dim; ++k) pts[i * dim + k] = coords[i + static_cast<size_t>(dim - 1 - k) * npts];
    intp_table* t = nullptr;
    intp_status st = intp_table_create(&desc, &t);
    if (st == INTP_OK) st = intp_table_interpolate(t, mesh, 0, nullptr);
    if (st == INTP_OK && npts > 0)
        st = intp_eval_host(t, pts.data(), static_cast<int64_t>(npts), deriv.data(), 1, result, INTP_F64, nullptr);
    std::string err = st == INTP_OK ? std::string() : std::string(intp_last_error());
    if (t) intp_table_destroy(t);
    return err;
}

}  // namespace intp_matlab
