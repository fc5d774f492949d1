// Batched line-solve kernels, element type DW (one instance per band class).
#include "batch_solve_impl.cuh"

INTP_DEFINE_BATCH_SOLVE(DW, dw)
