// C entry over the MATLAB binding's core (bsplineinterpolation_gb300/matlab/
// bspline_gpu_core.hpp) for the tests: the same MATLAB-layout arguments,
// called through ctypes. Returns 0 on success, else 1 with the reason in err.
#include <cstring>

#include "bspline_gpu_core.hpp"

extern "C" int mex_core_eval(uint64_t order, int dim, const unsigned char* periodic, const double* range,
                             const double* mesh, const uint64_t* dims, const double* coords, uint64_t npts,
                             const uint64_t* derivative, double* result, char* err, int errlen) {
    bool per[INTP_GPU_MAX_DIM] = {false, false, false, false};
    size_t d[INTP_GPU_MAX_DIM] = {0, 0, 0, 0};
    for (int j = 0; j < dim && j < INTP_GPU_MAX_DIM; ++j) {
        per[j] = periodic[j] != 0;
        d[j] = static_cast<size_t>(dims[j]);
    }
    const std::string e = intp_matlab::bspline_eval(order, dim, per, range, mesh, d, coords,
                                                    static_cast<size_t>(npts), derivative, result);
    if (e.empty()) return 0;
    std::strncpy(err, e.c_str(), static_cast<size_t>(errlen - 1));
    err[errlen - 1] = '\0';
    return 1;
}
