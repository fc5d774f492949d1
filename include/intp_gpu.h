/*
 * intp_gpu.h -- C ABI of the GB300-native B-spline interpolation library.
 *
 * Plain pointers and sizes only. Every call returns an intp_status; on failure
 * intp_last_error() describes the cause (thread-local). Device pointers are
 * CUDA global-memory pointers on the table's device; `stream` is a
 * cudaStream_t passed as void* (NULL = the default stream).
 *
 * The entry points replace the hot path of the header-only C++ reference
 * library 12ff54e/BSplineInterpolation (src/include/). Each declaration names
 * the reference interface it stands in for. Semantics are those of the
 * reference built with INTP_PERIODIC_NO_DUMMY_POINT: a periodic axis of n
 * samples has n control points and one period spans its range.
 */
#ifndef INTP_GPU_H
#define INTP_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define INTP_GPU_MAX_DIM 4
#define INTP_GPU_MAX_ORDER 7
#define INTP_GPU_MAX_DERIV 16

typedef enum intp_status {
    INTP_OK = 0,
    INTP_ERR_INVALID_ARGUMENT = 1, /* reference: INTP_ASSERT -> std::runtime_error */
    INTP_ERR_DOMAIN = 2,           /* reference: std::domain_error (range check) */
    INTP_ERR_OUT_OF_MEMORY = 3,    /* reference: std::bad_alloc */
    INTP_ERR_CUDA = 4,             /* CUDA runtime failure */
    INTP_ERR_STATE = 5,            /* e.g. evaluation before control points exist */
    INTP_ERR_UNSUPPORTED = 6,      /* dimension / order outside the compiled set */
    INTP_ERR_TIMEOUT = 7,          /* a bounded wait ran out */
    INTP_ERR_BUDGET = 8            /* serving: request exceeds the memory budget */
} intp_status;

typedef enum intp_precision {
    INTP_PRECISION_FP64 = 0,  /* FP64 end to end (parity form) */
    INTP_PRECISION_MIXED = 1  /* double-word (FP32-pair) solve, FP32 basis/contraction */
} intp_precision;

typedef enum intp_dtype { INTP_F64 = 0, INTP_F32 = 1 } intp_dtype;

typedef struct intp_table intp_table;
typedef struct intp_bandlu intp_bandlu;

/* Description of one interpolation table (one InterpolationFunction). */
typedef struct intp_table_desc {
    int32_t dim;           /* 1..INTP_GPU_MAX_DIM */
    int32_t order;         /* 0..INTP_GPU_MAX_ORDER */
    int32_t precision;     /* intp_precision */
    int32_t refine_steps;  /* mixed only: 0 = plain FP32 solve (FP32 control points); any other
                              value (default -1) = double-word solve (control points as FP32 pairs,
                              about 48 bits) */
    int32_t periodic[INTP_GPU_MAX_DIM];
    int64_t size[INTP_GPU_MAX_DIM];     /* samples per axis (mesh dim sizes) */
    double range_lo[INTP_GPU_MAX_DIM];  /* uniform axis: x_min */
    double range_hi[INTP_GPU_MAX_DIM];  /* uniform axis: x_max */
    /* non-uniform axis: host array of size[d] (+1 if periodic) increasing
     * sample coordinates; NULL for a uniform axis */
    const double* coords[INTP_GPU_MAX_DIM];
    /* values per mesh point: 0 or 1 = scalar table; C > 1 = vector-valued
     * table (the reference's InterpolationFunction<T, D, O> with a vector
     * type T, Interpolation.hpp:17-507). Values and control points are then
     * prod(size) x C, channel fastest, and every evaluation output is C
     * values. All channels share the knots, the factors and, per query, the
     * basis weights. Single tables (direct and binned evaluation), batches
     * and the serving loop take them; intp_eval_noalloc evaluates them with
     * the direct kernel. */
    int32_t channels;
    int32_t reserved_;
} intp_table_desc;

#define INTP_GPU_MAX_CHANNELS 64

/* Knot vectors, collocation matrices and their band LU factors, uploaded to
 * the current device.
 * Replaces: InterpolationFunctionTemplate::InterpolationFunctionTemplate
 * (src/include/InterpolationTemplate.hpp:60-79), which builds the knots
 * (src/include/Interpolation.hpp:322-464) and factors every axis
 * (InterpolationTemplate.hpp:254-446). */
intp_status intp_table_create(const intp_table_desc* desc, intp_table** out);

/* Releases the table and its device memory. Replaces the destructor of
 * InterpolationFunction / InterpolationFunctionTemplate. */
intp_status intp_table_destroy(intp_table* table);

/* Solves for control points from a row-major value mesh of prod(size)
 * doubles (host or device memory).
 * Replaces: InterpolationFunctionTemplate::interpolate
 * (InterpolationTemplate.hpp:118-143) -> solve_for_control_points_ (:448-580). */
intp_status intp_table_interpolate(intp_table* table, const double* values,
                                   int32_t values_on_device, void* stream);

/* Loads / reads control points (row-major, prod(size) doubles, host memory).
 * A mixed-precision table keeps every control point as a double-word (an
 * FP32 value plus its FP32 remainder, about 48 significant bits); one built
 * with refine_steps = 0 keeps the FP32 value alone.
 * Replaces: BSpline::load_ctrlPts (src/include/BSpline.hpp:230-242) and
 * BSpline::control_points (BSpline.hpp:575-577, plain layout). */
intp_status intp_table_set_control_points(intp_table* table, const double* ctrl_host);
intp_status intp_table_get_control_points(const intp_table* table, double* ctrl_host);

/* Axis properties. Replaces InterpolationFunction::periodicity / uniform /
 * range (Interpolation.hpp:248-258) and BSpline::knots_num (BSpline.hpp:592). */
intp_status intp_table_axis_info(const intp_table* table, int32_t axis, int64_t* nknots,
                                 double* range_lo, double* range_hi, int32_t* periodic,
                                 int32_t* uniform);
/* Copies the knot vector of one axis to host memory.
 * Replaces BSpline::knots_begin/knots_end (BSpline.hpp:560-571). */
intp_status intp_table_knots(const intp_table* table, int32_t axis, double* knots_host);

/* Batched evaluation at npts points (coords: npts x dim doubles, row-major,
 * device memory). derivs: nderiv x dim derivative orders (host memory), or
 * NULL for the value only (nderiv ignored, one output). out: npts x nderiv
 * values of out_dtype (device memory), row-major.
 * Replaces: InterpolationFunction::operator() (Interpolation.hpp:132-146) and
 * InterpolationFunction::derivative (Interpolation.hpp:177-205), i.e.
 * BSpline::operator() (BSpline.hpp:305-368) and BSpline::derivative_at
 * (BSpline.hpp:393-532), one call for many points. Out-of-range points on a
 * non-periodic axis extrapolate, as operator() does. */
intp_status intp_eval(const intp_table* table, const double* coords, int64_t npts,
                      const int32_t* derivs, int32_t nderiv, void* out, int32_t out_dtype,
                      void* stream);

/* As intp_eval with host buffers: the coordinates are copied to the device,
 * evaluated, and the results copied back before the call returns. Large
 * batches run as a pipeline of chunks (copy in, evaluate, copy out on three
 * streams). The coordinates are read from coords_host as it is when the call
 * is made: their copies do not wait for work queued earlier on `stream` (so
 * they overlap, e.g., a solve of the table just queued there), while every
 * evaluation does. Host memory from intp_host_alloc gives the full link
 * rate. */
intp_status intp_eval_host(const intp_table* table, const double* coords_host, int64_t npts,
                           const int32_t* derivs, int32_t nderiv, void* out_host,
                           int32_t out_dtype, void* stream);

/* ---- evaluation proxies ----
 *
 * Knot spans and basis weights of npts points (coords: npts x dim doubles,
 * device memory), computed once with `table`'s knots and kept in device
 * memory; intp_proxy_eval then evaluates any list of tables that share
 * those knots (same dimension, order, precision, periodicity and knot
 * vectors: tables built from one template) at all the points, value only.
 * Each value equals what intp_eval's direct path returns for that table.
 * Scalar tables of dimension 1..3.
 * Replaces: InterpolationFunctionTemplate::eval_proxy
 * (InterpolationTemplate.hpp:145-176), InterpolationFunction::eval_proxy
 * (Interpolation.hpp:493-503) and BSpline::pre_calc_coef (BSpline.hpp:
 * 250-296), which precompute one point's basis for reuse across functions. */
typedef struct intp_proxy intp_proxy;
intp_status intp_proxy_create(const intp_table* table, const double* coords, int64_t npts, void* stream,
                              intp_proxy** out);
intp_status intp_proxy_destroy(intp_proxy* proxy);
/* out: npts x ntables values of out_dtype (device memory), point-major:
 * out[i * ntables + j] = table j at point i. A table whose knots differ from
 * the proxy's fails with INTP_ERR_INVALID_ARGUMENT. */
intp_status intp_proxy_eval(const intp_proxy* proxy, const intp_table* const* tables, int32_t ntables, void* out,
                            int32_t out_dtype, void* stream);

/* Allocation-free form of intp_eval. No counterpart in the reference, whose
 * evaluation is per point on the host and needs no scratch.
 *
 * Same arguments and results as intp_eval, within FP32 rounding of each
 * output's scale. It allocates nothing on the device or the host: the
 * bucket-sort scratch of the binned path is one fixed 8 MiB device array
 * inside this library.
 *
 * Intended callers are those that cannot allocate while they evaluate:
 *  - a serving loop whose per-request latency must not include pool growth,
 *    or the device-wide synchronisation of cudaMalloc/cudaFree;
 *  - a process that has handed nearly all device memory to its own pool,
 *    where a scratch allocation could fail in the middle of a request.
 *
 * Requirements and limits:
 *  - The table's device must be current.
 *  - The first call on a device, whatever its table and point count,
 *    looks up the array's device address (cudaGetSymbolAddress), which may
 *    run the CUDA runtime's module set-up. Make that first call (npts = 0
 *    will do) before any stream capture.
 *  - The array is shared by every call on a device. Calls whose work
 *    overlaps on the device (several streams or host threads) race on it, so
 *    issue them on one stream. Its contents between calls do not matter:
 *    every word a call reads, the same call wrote earlier.
 *  - A table whose bucket bookkeeping leaves room for fewer than 1024 query
 *    records in the 8 MiB is rejected with INTP_ERR_INVALID_ARGUMENT (about
 *    32k buckets, e.g. a 512^3 cubic table); use intp_eval for it.
 *  - The number of points is not limited: they are taken in chunks that fit.
 *  - Tables outside the binned path (FP64 precision, dim 4, vector-valued
 *    tables) and batches below 2^18 points run the direct kernel, which
 *    needs no scratch. */
intp_status intp_eval_noalloc(const intp_table* table, const double* coords, int64_t npts,
                              const int32_t* derivs, int32_t nderiv, void* out, int32_t out_dtype,
                              void* stream);

/* Range check of InterpolationFunction::at / derivative_at
 * (Interpolation.hpp:153-169, :213-244, boundary_check_ :482-491) for a batch
 * of device coordinates: *first_bad = index of the first point outside the
 * range of a non-periodic axis, or -1. */
intp_status intp_check_range(const intp_table* table, const double* coords, int64_t npts,
                             int64_t* first_bad, void* stream);

/* Knot-span index per point and axis (npts x dim int64, device memory) and the
 * periodic-wrapped coordinate (npts x dim doubles, device memory, may be NULL).
 * Replaces BSpline::get_knot_iter (BSpline.hpp:125-157). */
intp_status intp_locate(const intp_table* table, const double* coords, int64_t npts,
                        int64_t* cells, double* wrapped, void* stream);

/* Knot-span index per point and axis (npts x dim int64, device memory) as the
 * binned evaluation computes it: the binned path's own locate kernel runs on
 * the points and its sort records are decoded. Mixed-precision scalar tables
 * of dimension 1..3 only (the tables intp_eval bins); INTP_ERR_UNSUPPORTED
 * otherwise. Diagnostics: it lets a caller check the binned path's spans
 * against BSpline::get_knot_iter (BSpline.hpp:125-157) point for point. */
intp_status intp_locate_binned(const intp_table* table, const double* coords, int64_t npts,
                               int64_t* cells, void* stream);

/* ---- diagnostics (failure paths) ----
 * No counterpart in the reference. They let a test drive the library's
 * failure paths without faulting or hanging the device. */

/* The binned evaluation waits for each staged tile on a barrier with a
 * bounded wait, and when the wait runs out it records INTP_ERR_TIMEOUT (read
 * by intp_stream_synchronize) and stops its work, after letting the copy in
 * flight land. probes > 0 replaces that wait by `probes` non-blocking tests
 * of the barrier, so that it runs out at once; 0 restores the normal wait.
 * Device-wide; for tests only. */
intp_status intp_debug_set_wait_limit(uint32_t probes);
/* Long mesh lines (single tables with few lines, and batched 1D tables)
 * are solved by a warp each: every lane takes a segment, starts a warm-up
 * of up to 64 (FP32) or 128 (FP64) rows before it from a zero state,
 * checks bit for bit that the warm-up reached its neighbour's values, and
 * is recomputed from them where it did not, so the control points equal a
 * serial sweep's. rows >= 0 caps the warm-up at `rows` (0: every segment
 * but the first is recomputed); -1 restores it. Device-wide; for tests
 * only. */
intp_status intp_debug_set_segment_warmup(int32_t rows);
/* Fails the next `count` device allocations of table storage (creation,
 * including tables built by the serving loop) as out of memory
 * (INTP_ERR_OUT_OF_MEMORY, the reference's std::bad_alloc) without calling
 * the allocator; 0 clears it. Process-wide; for tests only. */
intp_status intp_debug_fail_allocations(int32_t count);

/* Waits for `stream`. */
intp_status intp_stream_synchronize(void* stream);

/* Page-locked host memory for the host-buffer entry points
 * (intp_eval_host, intp_table_interpolate with host values): allocated by
 * the CUDA runtime's own host allocator, so copies between it and the device
 * run at the full host link rate. No counterpart in the reference, whose data
 * never leaves host memory. intp_host_free releases it. */
intp_status intp_host_alloc(size_t bytes, void** ptr);
intp_status intp_host_free(void* ptr);

/* Description of the last failure on the calling thread. */
const char* intp_last_error(void);

/* Number of CUDA kernels the library has launched in this process
 * (diagnostic; no counterpart in the reference). */
uint64_t intp_launch_count(void);

/* ---- batched tables ----
 *
 * Many independent tables (InterpolationFunction objects of uneven size,
 * order, periodicity and dimension 1..3) built and evaluated together: one
 * device arena for all knots and factors, one control-point array, and one
 * launch per axis pass (solve) or per (dimension, order) class (evaluation)
 * for the whole batch. The reference builds and evaluates such tables one
 * object at a time; a batched table's control points and values are those of
 * the same table built alone with intp_table_create/intp_table_interpolate
 * and evaluated with intp_eval's direct kernel, bit for bit. */
typedef struct intp_batch intp_batch;

/* Knots and factors of ntables tables (descs[i], all of one precision) on the
 * current device. Replaces ntables InterpolationFunctionTemplate
 * constructions (InterpolationTemplate.hpp:60-79). */
intp_status intp_batch_create(const intp_table_desc* descs, int64_t ntables, intp_batch** out);
intp_status intp_batch_destroy(intp_batch* batch);
/* Number of tables and total number of mesh values (sum of prod(size) x C). */
intp_status intp_batch_info(const intp_batch* batch, int64_t* ntables, int64_t* total_values);

/* Solves the control points of every table. `values` holds each table's
 * row-major value mesh, in table order (total_values doubles, host or device
 * memory; a C-channel table's C values per mesh point consecutive). Replaces InterpolationFunctionTemplate::interpolate
 * (InterpolationTemplate.hpp:118-143) once per table. */
intp_status intp_batch_build(intp_batch* batch, const double* values, int32_t values_on_device, void* stream);

/* Schedule of a batch's line solves. No counterpart in the reference, whose
 * tables build one by one on its thread pool (InterpolationTemplate.hpp:
 * 547-569). None of the choices changes the arithmetic of any line: every
 * schedule gives the same control points, bit for bit. */
typedef struct intp_batch_schedule {
    int32_t persistent;    /* 1: each axis pass is a grid of a few warps per SM draining an atomic work
                              queue (longest lines first); 0: one CTA per work item */
    int32_t contig_rows;   /* lines per work item on the contiguous axis (1..32); each chunk of them
                              moves through a per-warp shared-memory transpose */
    int32_t strided_rows;  /* lines per work item on strided axes (1..32) */
    int32_t pad_;
    double build_ms;       /* build time measured by intp_batch_autotune (0 when set by hand) */
} intp_batch_schedule;

/* Sets / reads the schedule (the default: one CTA per item, 32 lines per item on every axis). */
intp_status intp_batch_set_schedule(intp_batch* batch, const intp_batch_schedule* schedule);
intp_status intp_batch_get_schedule(const intp_batch* batch, intp_batch_schedule* schedule);
/* Times a build of the batch from `values` (as intp_batch_build) under each
 * candidate schedule, keeps the fastest, records its time in build_ms, and
 * leaves the batch built under it (*chosen may be NULL). */
intp_status intp_batch_autotune(intp_batch* batch, const double* values, int32_t values_on_device,
                                void* stream, intp_batch_schedule* chosen);

/* Control points of one table (prod(size) x C doubles, channel fastest, host
 * memory).
 * Replaces BSpline::control_points (BSpline.hpp:575-577). */
intp_status intp_batch_get_control_points(const intp_batch* batch, int64_t table, double* ctrl_host);

/* Evaluates every table at its own points. point_offsets (host memory,
 * ntables + 1 entries, point_offsets[0] = 0) gives table i the points
 * point_offsets[i] .. point_offsets[i+1]-1; coords (device memory) holds
 * those points table after table, dim_i doubles per point. derivs (host
 * memory): nderiv rows of INTP_GPU_MAX_DIM orders, of which a table of
 * dimension D uses the first D, or NULL for the value only. out (device
 * memory): table after table, each table's points x nderiv x C values of
 * out_dtype (C = 1 for scalar tables: point_offsets[ntables] x nderiv in
 * all for a scalar batch).
 * Replaces InterpolationFunction::operator() / derivative
 * (Interpolation.hpp:132-146, :177-205) per table and point. */
intp_status intp_batch_eval(const intp_batch* batch, const double* coords, const int64_t* point_offsets,
                            const int32_t* derivs, int32_t nderiv, void* out, int32_t out_dtype, void* stream);

/* A CUDA graph of one build and one evaluation of the batch: the arguments
 * of intp_batch_build (device values) and intp_batch_eval, fixed at
 * creation. Creation builds the batch once, uploads the evaluation's work
 * list, then captures the build's launches (on side streams too) and the
 * evaluation's launches. intp_batch_graph_launch replays them on `stream`,
 * reading the values and coordinates then in those buffers; results equal
 * those of intp_batch_build + intp_batch_eval on the same contents, bit for
 * bit. The graph keeps pointers to the batch and the buffers: destroy it
 * first. A new schedule (intp_batch_set_schedule, intp_batch_autotune)
 * replaces the work lists the graph reads: its launches then fail with
 * INTP_ERR_STATE. No counterpart in the reference. */
typedef struct intp_batch_graph intp_batch_graph;
intp_status intp_batch_graph_create(intp_batch* batch, const double* values, const double* coords,
                                    const int64_t* point_offsets, const int32_t* derivs, int32_t nderiv, void* out,
                                    int32_t out_dtype, intp_batch_graph** out_graph);
intp_status intp_batch_graph_launch(intp_batch_graph* graph, void* stream);
intp_status intp_batch_graph_destroy(intp_batch_graph* graph);

/* ---- serving loop ----
 *
 * A worker thread that keeps built tables resident in device memory and
 * runs table-build and evaluate requests with continuous batching: requests
 * submitted while others run are admitted as soon as a slot (a CUDA stream)
 * and memory free up, their work overlaps on the device, and evaluations
 * queued against the same table are merged into one launch. Resident tables
 * plus in-flight work stay within a memory budget; least recently used idle
 * tables are evicted to make room. The reference has no server: a request
 * stands for constructing an InterpolationFunction (Interpolation.hpp:92-107)
 * or calling its operator() / derivative (:132-146, :177-205) on many points.
 *
 * Host buffers passed to the submit calls (values, coordinates, outputs) must
 * stay valid until intp_server_wait reports the request done; page-locked
 * host memory (or device memory) lets the copies run asynchronously. */
typedef struct intp_server intp_server;

typedef struct intp_server_config {
    uint64_t memory_budget;    /* device bytes for tables + work in flight; 0 = 150 GiB */
    int32_t slots;             /* work units in flight (CUDA streams), 1..64; 0 = 4 */
    int32_t pad_;
    int64_t max_batch_points;  /* merged evaluation size limit; 0 = 2^24 points */
} intp_server_config;

typedef struct intp_server_stats {
    int64_t builds_done, evals_done, failed, evictions, merged_units, resident_tables;
    uint64_t resident_bytes, inflight_bytes;
    double points_evaluated;
    double build_p50_ms, build_p99_ms, eval_p50_ms, eval_p99_ms, all_p50_ms, all_p99_ms;
    double points_per_s;  /* points evaluated since the last reset / time to the last completion */
} intp_server_stats;

/* Table states reported by intp_server_table_state. */
#define INTP_SERVER_TABLE_QUEUED 0
#define INTP_SERVER_TABLE_RESIDENT 1
#define INTP_SERVER_TABLE_GONE 2   /* evicted or released */
#define INTP_SERVER_TABLE_FAILED 3

/* Starts the worker on the current device (cfg may be NULL for defaults).
 * The server reserves min(memory_budget, 64 GiB) in the device's
 * stream-ordered memory pool up front (the pool then keeps freed memory), so
 * that admitting a request does not wait for new device memory to be
 * mapped. */
intp_status intp_server_create(const intp_server_config* cfg, intp_server** out);
/* Finishes every submitted request, then frees the tables and the worker. */
intp_status intp_server_destroy(intp_server* server);

/* Queues the build of one table from its value mesh (prod(size) doubles,
 * host or device memory): a new table id, usable by evaluations at once
 * (they run after the build). Replaces constructing an InterpolationFunction
 * (Interpolation.hpp:92-107). */
intp_status intp_server_submit_build(intp_server* server, const intp_table_desc* desc, const double* values,
                                     int64_t* table_id, int64_t* request_id);
/* Queues an evaluation of npts points (npts x dim doubles) of a table, with
 * the derivs / nderiv / out_dtype meaning of intp_eval; out receives
 * npts x nderiv values (host or device memory). Replaces
 * InterpolationFunction::operator() / derivative (Interpolation.hpp:132-146,
 * :177-205) on each point. */
intp_status intp_server_submit_eval(intp_server* server, int64_t table_id, const double* coords, int64_t npts,
                                    const int32_t* derivs, int32_t nderiv, void* out, int32_t out_dtype,
                                    int64_t* request_id);
/* Waits up to timeout_s seconds (< 0: no limit) for a request; *result is
 * its status (INTP_ERR_BUDGET: it can never fit the budget; INTP_ERR_STATE:
 * its table was evicted, released or failed to build). Each request is
 * waited on once. INTP_ERR_TIMEOUT: still running. */
intp_status intp_server_wait(intp_server* server, int64_t request_id, double timeout_s, intp_status* result);
/* Drops a table once the requests that use it are done. */
intp_status intp_server_release(intp_server* server, int64_t table_id);
/* One of INTP_SERVER_TABLE_*. */
intp_status intp_server_table_state(intp_server* server, int64_t table_id, int32_t* state);
/* Latency percentiles and throughput since the last reset. */
intp_status intp_server_get_stats(intp_server* server, intp_server_stats* out);
intp_status intp_server_reset_stats(intp_server* server);

/* ---- standalone band LU (BandLU.hpp) ---- */

/* Factors an n x n band matrix given in the reference's storage: band is
 * n x (1+p+q) with A(i,j) = band[j*(1+p+q) + (i+q-j)]; cyclic matrices add
 * right ((n-q-1) x p, R(i, j+p-n)) and bottom ((n-p-1) x q, S(j, i+q-n))
 * corner blocks (NULL when cyclic == 0). Only p == q is supported.
 * Replaces: BandLU<BandMatrix>::compute (src/include/BandLU.hpp:31-41,
 * :103-118) and BandLU<ExtendedBandMatrix>::compute (:159-213). */
intp_status intp_bandlu_create(int64_t n, int32_t p, int32_t q, int32_t cyclic, const double* band,
                               const double* right, const double* bottom, intp_bandlu** out);
/* Solves in place along the middle axis of an (outer, n, inner) row-major
 * tensor of doubles in device memory.
 * Replaces: BandLU::solve_in_place (BandLU.hpp:51-54, :120-143, :215-259). */
intp_status intp_bandlu_solve(const intp_bandlu* lu, double* x, int64_t outer, int64_t inner,
                              void* stream);
intp_status intp_bandlu_destroy(intp_bandlu* lu);

#ifdef __cplusplus
}
#endif

#endif /* INTP_GPU_H */
