// Batched line-solve kernels, element type double (one instance per band class).
#include "batch_solve_impl.cuh"

INTP_DEFINE_BATCH_SOLVE(double, f64)
