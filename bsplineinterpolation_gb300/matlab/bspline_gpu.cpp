// MATLAB MEX gateway over the GPU library, a drop-in for the reference's
// matlab/bspline.cpp (same name of arguments, same order and types, same
// checks and messages):
//
//   result = bspline_gpu(uint64(order), is_periodic, range, mesh, coords, uint64(derivative))
//
// Build (MATLAB's mex with this repository's include/ directory and the
// CUDA library):
//   mex -I<repo>/include -I<repo>/bsplineinterpolation_gb300/matlab ...
//       -L<repo>/bsplineinterpolation_gb300 -lintp_gb300 bspline_gpu.cpp
// The C MEX API is used (mex.h), so any MATLAB release builds it.
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "bspline_gpu_core.hpp"
#include "mex.h"

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
    (void)nlhs;
    if (nrhs != 6) mexErrMsgIdAndTxt("bspline_gpu:args", "Six input required");
    if (!mxIsUint64(prhs[0]) || !mxIsLogical(prhs[1]) || !mxIsDouble(prhs[2]) || !mxIsDouble(prhs[3]) ||
        !mxIsDouble(prhs[4]) || !mxIsUint64(prhs[5]))
        mexErrMsgIdAndTxt("bspline_gpu:type", "Input type error");
    const uint64_t order = static_cast<const uint64_t*>(mxGetData(prhs[0]))[0];
    const mxArray* mesh = prhs[3];
    const size_t nd = mxGetNumberOfDimensions(mesh);
    const size_t* md = mxGetDimensions(mesh);
    std::vector<size_t> dims;
    for (size_t i = 0; i < nd; ++i)
        if (md[i] > 1) dims.push_back(md[i]);
    const int dim = static_cast<int>(dims.size());
    const mxArray* range = prhs[2];
    if (mxGetNumberOfDimensions(range) != 2 || mxGetM(range) != static_cast<size_t>(dim) || mxGetN(range) != 2)
        mexErrMsgIdAndTxt("bspline_gpu:range", "Range require Dim * 2 array");
    if (md[0] == 1) mexErrMsgIdAndTxt("bspline_gpu:mesh", "Mesh should be col vector for 1 dimension");
    if (mxGetNumberOfElements(prhs[1]) != static_cast<size_t>(dim) ||
        mxGetNumberOfElements(prhs[5]) != static_cast<size_t>(dim))
        mexErrMsgIdAndTxt("bspline_gpu:args", "is_periodic, derivative_in require length dim array");
    const mxArray* coords = prhs[4];
    if (mxGetNumberOfDimensions(coords) != 2 || mxGetN(coords) != static_cast<size_t>(dim))
        mexErrMsgIdAndTxt("bspline_gpu:coords", "Interpolate coordinate require N * dim array");
    const size_t npts = mxGetM(coords);
    const mxLogical* per = mxGetLogicals(prhs[1]);
    bool pb[INTP_GPU_MAX_DIM] = {false, false, false, false};
    for (int j = 0; j < dim && j < INTP_GPU_MAX_DIM; ++j) pb[j] = per[j] != 0;
    plhs[0] = mxCreateDoubleMatrix(npts, 1, mxREAL);
    const std::string err = intp_matlab::bspline_eval(
        order, dim, pb, mxGetPr(range), mxGetPr(mesh), dims.data(), mxGetPr(coords), npts,
        static_cast<const uint64_t*>(mxGetData(prhs[5])), mxGetPr(plhs[0]));
    if (!err.empty()) mexErrMsgIdAndTxt("bspline_gpu:eval", "%s", err.c_str());
}
