// Table operations used inside the library beyond the C-ABI (the serving
// loop, server.cu); defined in capi.cu.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "intp_gpu.h"

namespace intp_gb300 {

// intp_table_create, optionally with every device allocation of the table
// taken from the stream-ordered pool on `stream` (and freed there).
intp_status create_table(const intp_table_desc* desc, bool stream_ordered, cudaStream_t stream, intp_table** out);

// Device bytes a table holds now (per-axis arena, control points, solve
// scratch).
size_t table_device_bytes(const intp_table* t);

// Upper bound of the transient device bytes of one intp_table_interpolate of
// a table with this description (values staging and refinement buffers).
size_t table_build_scratch_bytes(const intp_table_desc* desc);

// Frees the solve scratch (kept by default for the next interpolate).
void table_release_scratch(intp_table* t);

// Number of control points (product of the axis sizes).
int64_t table_values(const intp_table* t);

// Keeps memory freed to the current device's stream-ordered pool in the pool
// (no release back to the driver at synchronisation points); once per process.
void retain_pool_memory();

}  // namespace intp_gb300
