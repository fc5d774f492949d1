/* Declarations of the C MEX API functions the MATLAB gateway uses, with the
 * signatures of MATLAB's mex.h / matrix.h: enough to compile-check the
 * gateway without MATLAB (nothing here is linked or run). */
#pragma once
#include <cstddef>
typedef struct mxArray_tag mxArray;
typedef bool mxLogical;
typedef enum { mxREAL, mxCOMPLEX } mxComplexity;
bool mxIsUint64(const mxArray*);
bool mxIsLogical(const mxArray*);
bool mxIsDouble(const mxArray*);
void* mxGetData(const mxArray*);
double* mxGetPr(const mxArray*);
mxLogical* mxGetLogicals(const mxArray*);
size_t mxGetNumberOfDimensions(const mxArray*);
const size_t* mxGetDimensions(const mxArray*);
size_t mxGetNumberOfElements(const mxArray*);
size_t mxGetM(const mxArray*);
size_t mxGetN(const mxArray*);
mxArray* mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity flag);
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
