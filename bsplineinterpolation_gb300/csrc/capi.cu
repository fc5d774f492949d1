// C-ABI of the library (include/intp_gpu.h): table lifetime, the control-point
// solve pipelines and batched evaluation.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "intp_gpu.h"
#include "launch.hpp"
#include "spline_model.hpp"
#include "table_internal.hpp"
#include "table_pack.hpp"

using namespace intp_gb300;

namespace {

std::atomic<unsigned long long> g_launches{0};
// Diagnostics (intp_debug_fail_allocations): device allocations of tables
// still to be failed as out of memory, without calling the allocator.
std::atomic<int> g_fail_allocs{0};

bool take_injected_alloc_failure() {
    int v = g_fail_allocs.load();
    while (v > 0)
        if (g_fail_allocs.compare_exchange_weak(v, v - 1)) return true;
    return false;
}

// binned evaluation: queries per chunk. Each bucket's tile is staged once per
// evaluation CTA that meets the bucket, so more queries per sort share each
// staged tile; but the scatter spreads its records over the whole chunk's
// record array, and it slows down as that grows. 2^25 queries measured best
// on the 3D cubic 256^3 workload (2^23: evaluation slower; 2^28: scatter
// slower).
constexpr int64_t kDefaultChunk = int64_t{1} << 25;
// host-buffer evaluation (intp_eval_host): the largest chunk of its copy-in
// / evaluate / copy-out pipeline, its first chunk (the copy-in that nothing
// overlaps; chunks double from it), and the device buffers of each kind in
// the ring. The host link bounds the pipeline, so small chunks cost little
// evaluation rate and shorten the evaluation and copy-out left after the
// last copy-in: 2^22 points measured best on the 3D cubic 256^3 workload
// (1e8 points: 13.15 ms, against 13.35 at 2^23 and 13.97 at 2^25).
constexpr int64_t kHostPipelineChunk = int64_t{1} << 22;
constexpr int64_t kHostHeadChunk = int64_t{1} << 21;
constexpr int kHostBuffers = 3;
// the smallest batch worth binning
constexpr int64_t kBinnedMinPoints = int64_t{1} << 18;

// INTP_GB300_EVAL = direct | binned | auto (default); INTP_GB300_CHUNK = queries per chunk
int eval_mode() {
    const char* v = std::getenv("INTP_GB300_EVAL");
    if (!v) return 0;
    if (std::strcmp(v, "direct") == 0) return 1;
    if (std::strcmp(v, "binned") == 0) return 2;
    return 0;
}

int64_t eval_chunk() {
    const char* v = std::getenv("INTP_GB300_CHUNK");
    if (!v) return kDefaultChunk;
    const long long c = std::atoll(v);
    // a record holds its query's index within a sort CTA's slice in 20 bits
    return c >= 1024 ? std::min<long long>(c, int64_t{1} << 28) : kDefaultChunk;
}

}  // namespace

// Keep memory freed by cudaFreeAsync in the device's default pool so
// per-call scratch of the binned evaluation is reused, not re-mapped.
void intp_gb300::retain_pool_memory() {
    static std::atomic<bool> done{false};
    if (done.exchange(true)) return;
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thr = ~uint64_t{0};
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
}

namespace {

thread_local std::string g_last_error;

intp_status fail(intp_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

intp_status cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return INTP_ERR_OUT_OF_MEMORY;
    return INTP_ERR_CUDA;
}

#define INTP_CUDA(call, what)                            \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

std::vector<float> to_f32(const std::vector<double>& v) {
    std::vector<float> r(v.size());
    for (size_t i = 0; i < v.size(); ++i) r[i] = factor_f32(v[i]);
    return r;
}

std::vector<DW> to_dw(const std::vector<double>& v) {
    std::vector<DW> r(v.size());
    for (size_t i = 0; i < v.size(); ++i) r[i] = dw_from_double(v[i]);
    return r;
}

}  // namespace

struct intp_table {
    TableModel model;
    int channels = 1;  // values per mesh point (vector-valued tables)
    int precision = INTP_PRECISION_FP64;
    int refine_steps = 0;
    int device = 0;
    void* arena = nullptr;
    void* ctrl = nullptr;
    // refined mixed tables: the FP32 remainder of every control point
    // (control point = ctrl + ctrl_lo as a double-float), else null
    float* ctrl_lo = nullptr;
    bool has_ctrl = false;
    TableDev dev{};
    BinGeom bins{};
    AxisFactorDev fac[kMaxDim]{};
    void* scratch = nullptr;  // solve scratch (values staging, refinement buffers)
    size_t scratch_bytes = 0;
    double lo_user[kMaxDim]{};  // uniform axes: x_range.first
    size_t arena_bytes = 0;
    // TMA maps of the FP32 control points and of their remainders (when the
    // table keeps them) whose box is one bucket tile of the binned
    // evaluation (D = 2, 3 with 16-byte aligned row strides)
    CUtensorMap tile_map[2]{};
    bool has_tile_map = false;
    // Tables of the serving loop take their memory from the stream-ordered
    // pool on alloc_stream (no device-wide synchronisation on free).
    bool stream_ordered = false;
    cudaStream_t alloc_stream = nullptr;

    cudaError_t dmalloc(void** p, size_t bytes) {
        if (take_injected_alloc_failure()) return cudaErrorMemoryAllocation;
        return stream_ordered ? cudaMallocAsync(p, bytes, alloc_stream) : cudaMalloc(p, bytes);
    }
    void dfree(void* p) {
        if (!p) return;
        if (stream_ordered)
            cudaFreeAsync(p, alloc_stream);
        else
            cudaFree(p);
    }
    ~intp_table() {
        dfree(arena);
        dfree(ctrl);
        dfree(ctrl_lo);
        dfree(scratch);
    }
    bool mixed() const { return precision == INTP_PRECISION_MIXED; }
    // refinement steps of the mixed solve (the automatic choice resolved)
    // mixed form: 1 = the double-word solve (control points as FP32 pairs),
    // 0 = the plain FP32 solve (refine_steps = 0)
    int steps() const { return !mixed() ? 0 : refine_steps == 0 ? 0 : 1; }
    size_t elem() const { return mixed() ? sizeof(float) : sizeof(double); }
    int64_t values() const { return model.total * channels; }  // control points over all channels
};

// An evaluation proxy: the geometry it was built with (to check the tables it
// evaluates) and its per-point spans, offsets and weights in device memory.
struct intp_proxy {
    int device = 0;
    int precision = INTP_PRECISION_FP64;
    int dim = 0, order = 0;
    bool periodic[kMaxDim]{};
    std::vector<double> knots[kMaxDim];
    int64_t npts = 0;
    void* mem = nullptr;
    int64_t* cells = nullptr;
    void* xr = nullptr;
    void* base = nullptr;
    ~intp_proxy() {
        if (mem) cudaFree(mem);
    }
};

struct intp_bandlu {
    LineFactor f;
    void* arena = nullptr;
    const double *lower = nullptr, *upper = nullptr, *dinv = nullptr, *bottom = nullptr,
                 *right = nullptr;
    ~intp_bandlu() {
        if (arena) cudaFree(arena);
    }
};

namespace {

// cuTensorMapEncodeTiled from the driver, looked up through the runtime (the
// library links no driver library).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// A TMA map of the control points whose box is one bucket tile: extents P_d
// per axis, the last padded to a multiple of 4 floats. Positions past the end
// of a non-periodic axis read zeros (no query reads them). Needs row strides
// that are multiples of 16 bytes and boxes of at most 256 per axis.
bool make_tile_map(intp_table* t, void* base, CUtensorMap* map) {
    const TableModel& m = t->model;
    const BinGeom& g = t->bins;
    const int D = m.dim;
    if (D < 2 || D > 3) return false;
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return false;
    cuuint64_t dims[3] = {}, strides[2] = {};
    cuuint32_t box[3] = {}, estr[3] = {1, 1, 1};
    for (int i = 0; i < D; ++i) {
        const int d = D - 1 - i;  // innermost first
        dims[i] = static_cast<cuuint64_t>(m.axis[d].n);
        box[i] = static_cast<cuuint32_t>(i == 0 ? ((g.P[d] + 3) & ~3) : g.P[d]);
        if (box[i] > 256) return false;
    }
    strides[0] = static_cast<cuuint64_t>(m.axis[D - 1].n) * 4;
    if (D == 3) strides[1] = strides[0] * static_cast<cuuint64_t>(m.axis[1].n);
    for (int i = 0; i < D - 1; ++i)
        if (strides[i] % 16 != 0) return false;
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, static_cast<cuuint32_t>(D), base, dims,
                           strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// Per-axis tables used by evaluation and the solve, laid out in one arena.
intp_status upload_table(intp_table* t) {
    const TableModel& m = t->model;
    Arena ar;
    PackedTable pt;
    pack_table(m, ar, pt);
    INTP_CUDA(t->dmalloc(&t->arena, ar.host.size()), "cudaMalloc(table)");
    t->arena_bytes = ar.host.size();
    if (t->stream_ordered)
        INTP_CUDA(cudaMemcpyAsync(t->arena, ar.host.data(), ar.host.size(), cudaMemcpyHostToDevice, t->alloc_stream),
                  "cudaMemcpyAsync(table)");
    else
        INTP_CUDA(cudaMemcpy(t->arena, ar.host.data(), ar.host.size(), cudaMemcpyHostToDevice), "cudaMemcpy(table)");
    bind_table(m, t->lo_user, pt, static_cast<const unsigned char*>(t->arena), t->dev, t->fac);
    INTP_CUDA(t->dmalloc(&t->ctrl, static_cast<size_t>(t->values()) * t->elem()), "cudaMalloc(control points)");
    t->dev.ctrl = t->ctrl;
    if (t->steps() > 0) {
        INTP_CUDA(t->dmalloc(reinterpret_cast<void**>(&t->ctrl_lo), static_cast<size_t>(t->values()) * sizeof(float)),
                  "cudaMalloc(control point remainders)");
        t->dev.ctrl_lo = t->ctrl_lo;
    }
    t->dev.channels = t->channels;
    t->dev.chan_stride = m.total;
    // binned evaluation: a vector-valued table's channels are staged one
    // after another by element copies (the TMA maps cover one channel)
    if (t->mixed() && m.dim <= 3) {
        t->bins = make_bin_geom(t->dev);
        if (t->bins.smem_buckets > 0 && t->channels == 1)
            t->has_tile_map = make_tile_map(t, t->ctrl, &t->tile_map[0]) &&
                              (!t->ctrl_lo || make_tile_map(t, t->ctrl_lo, &t->tile_map[1]));
    }
    return INTP_OK;
}

intp_status ensure_scratch(intp_table* t, size_t bytes) {
    if (t->scratch_bytes >= bytes) return INTP_OK;
    t->dfree(t->scratch);
    t->scratch = nullptr;
    t->scratch_bytes = 0;
    INTP_CUDA(t->dmalloc(&t->scratch, bytes), "cudaMalloc(solve scratch)");
    t->scratch_bytes = bytes;
    return INTP_OK;
}

ShiftDesc shift_desc(const intp_table* t) {
    ShiftDesc sd{};
    const TableModel& m = t->model;
    sd.dim = m.dim;
    sd.total = m.total;
    sd.channels = t->channels;
    for (int d = 0; d < m.dim; ++d) {
        sd.n[d] = m.axis[d].n;
        sd.shift[d] = m.axis[d].periodic ? (m.order / 2) % m.axis[d].n : 0;
        sd.stride[d] = t->dev.ax[d].stride;
    }
    return sd;
}

struct LineGeom {
    int64_t n, S, nlines;
};

LineGeom line_geom(const intp_table* t, int axis) {
    const TableModel& m = t->model;
    LineGeom g;
    g.n = m.axis[axis].n;
    g.S = t->dev.ax[axis].stride;
    g.nlines = t->values() / g.n;  // every channel's lines (channel-major storage)
    return g;
}

cudaError_t solve_f32_all(intp_table* t, float* x, cudaStream_t s) {
    for (int a = t->model.dim - 1; a >= 0; --a) {
        const LineGeom g = line_geom(t, a);
        const AxisFactorDev& f = t->fac[a];
        const LineFactor& lf = t->model.axis[a].factor;
        cudaError_t e = launch_line_solve_f32(x, g.n, g.S, g.nlines, lf.p, lf.q, lf.cyclic, f.lowerf, f.upperf,
                                              f.dinvf, f.bottomf, f.rightf, s, f.clo32, f.chi32, f.zside32);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t solve_dw_all(intp_table* t, DW* x, cudaStream_t s) {
    for (int a = t->model.dim - 1; a >= 0; --a) {
        const LineGeom g = line_geom(t, a);
        const AxisFactorDev& f = t->fac[a];
        const LineFactor& lf = t->model.axis[a].factor;
        cudaError_t e = launch_line_solve_dw(x, g.n, g.S, g.nlines, lf.p, lf.q, lf.cyclic, f.lowerw, f.upperw, f.dinvw,
                                             f.bottomw, f.rightw, s, f.clo, f.chi, f.zside);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t solve_f64_all(intp_table* t, double* x, cudaStream_t s) {
    for (int a = t->model.dim - 1; a >= 0; --a) {
        const LineGeom g = line_geom(t, a);
        const AxisFactorDev& f = t->fac[a];
        const LineFactor& lf = t->model.axis[a].factor;
        cudaError_t e = launch_line_solve_f64(x, g.n, g.S, g.nlines, lf.p, lf.q, lf.cyclic, f.lower, f.upper,
                                              f.dinv, f.bottom, f.right, s, f.clo, f.chi, f.zside);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

intp_status run_interpolate(intp_table* t, const double* values_dev, cudaStream_t s) {
    const TableModel& m = t->model;
    const int64_t N = t->values();
    const ShiftDesc sd = shift_desc(t);
    if (!t->mixed()) {
        double* c = static_cast<double*>(t->ctrl);
        INTP_CUDA(launch_shift_copy_f64_f64(values_dev, c, sd, s), "shift copy");
        INTP_CUDA(solve_f64_all(t, c, s), "line solve (fp64)");
        t->has_ctrl = true;
        return INTP_OK;
    }
    float* c = static_cast<float*>(t->ctrl);
    const int steps = t->steps();
    if (steps == 0) {
        INTP_CUDA(launch_shift_copy_f64_f32(values_dev, c, nullptr, nullptr, sd, s), "shift copy");
        INTP_CUDA(solve_f32_all(t, c, s), "line solve (fp32)");
    } else {
        // Double-word solve: the shifted values split into double-words, one
        // band substitution per axis in double-word arithmetic (R = DW), the
        // solution split into the control points' two FP32 arrays.
        const size_t need = static_cast<size_t>(N) * sizeof(DW) + 1024;
        intp_status st = ensure_scratch(t, need);
        if (st != INTP_OK) return st;
        DW* w = static_cast<DW*>(t->scratch);
        INTP_CUDA(launch_shift_copy_f64_dw(values_dev, w, sd, s), "shift copy");
        INTP_CUDA(solve_dw_all(t, w, s), "line solve (double-word)");
        INTP_CUDA(launch_dw_unpack(w, c, t->ctrl_lo, N, s), "double-word split");
    }
    t->has_ctrl = true;
    return INTP_OK;
}

bool make_plan(const intp_table* t, const int32_t* derivs, int32_t nderiv, DerivPlan& plan,
               std::string& err) {
    return build_deriv_plan(t->model.dim, t->model.order, derivs, nderiv, t->model.dim, plan, err);
}

// ---- fixed scratch of the allocation-free evaluation (intp_eval_noalloc) ----
//
// One file-scope device array, the same on every device that loads this
// library (held until the process exits). In host code its name is only a
// host-side stand-in for the symbol, so the device address is looked up with
// cudaGetSymbolAddress, once per device, with that device current.
constexpr size_t kNoAllocScratchBytes = size_t{8} << 20;  // 8 MiB
constexpr int kNoAllocSortBlocks = 32;
constexpr int kNoAllocMaxDevices = 64;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
std::mutex g_noalloc_mutex;
void* g_noalloc_addr[kNoAllocMaxDevices] = {};

intp_status noalloc_scratch_address(int dev, void** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(INTP_ERR_UNSUPPORTED, "device ordinal out of range");
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)");
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return INTP_OK;
}

}  // namespace

namespace intp_gb300 {

void set_last_error(const std::string& msg) { g_last_error = msg; }

// Groups outputs by their derivative orders on axes 1..D-1.
void group_plan(DerivPlan& plan, int dim) {
    plan.ngroups = 0;
    for (int k = 0; k < plan.k; ++k) {
        int g = 0;
        for (; g < plan.ngroups; ++g) {
            bool same = true;
            for (int d = 1; d < dim; ++d) same = same && plan.ord[plan.group_rep[g]][d] == plan.ord[k][d];
            if (same) break;
        }
        if (g == plan.ngroups) plan.group_rep[plan.ngroups++] = static_cast<int8_t>(k);
        plan.out_group[k] = static_cast<int8_t>(g);
    }
    plan.simple = plan.ngroups == 1 ? 1 : 0;
    for (int d = 1; d < dim && plan.simple; ++d)
        if (plan.ord[plan.group_rep[0]][d] != 0) plan.simple = 0;
    plan.has_deriv = 0;
    for (int k = 0; k < plan.k; ++k)
        for (int d = 0; d < dim; ++d)
            if (plan.ord[k][d] != 0) plan.has_deriv = 1;
}

bool build_deriv_plan(int dim, int order, const int32_t* derivs, int32_t nderiv, int row_stride, DerivPlan& plan,
                      std::string& err) {
    std::memset(&plan, 0, sizeof plan);
    if (!derivs) {
        plan.k = 1;
        group_plan(plan, dim);
        return true;
    }
    if (nderiv < 1 || nderiv > kMaxDeriv) {
        err = "nderiv must be in [1, 16]";
        return false;
    }
    plan.k = nderiv;
    for (int k = 0; k < nderiv; ++k)
        for (int d = 0; d < dim; ++d) {
            const int32_t v = derivs[k * row_stride + d];
            if (v < 0) {
                err = "derivative orders must be non-negative";
                return false;
            }
            // any order above the spline order gives 0 (BSpline.hpp:404-407)
            plan.ord[k][d] = static_cast<int8_t>(std::min<int32_t>(v, order + 1));
        }
    group_plan(plan, dim);
    // second and higher derivatives of high-order tables: the precise mixed
    // contraction (the plain FP32 one leaves them near 2e-6 of their scale)
    for (int k = 0; k < plan.k; ++k)
        for (int d = 0; d < dim; ++d)
            if (order >= 4 && plan.ord[k][d] >= 2 && plan.ord[k][d] <= order) plan.precise = 1;
    return true;
}

intp_status create_table(const intp_table_desc* desc, bool stream_ordered, cudaStream_t stream, intp_table** out) {
    if (!desc || !out) return fail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (desc->dim < 1 || desc->dim > INTP_GPU_MAX_DIM)
        return fail(INTP_ERR_UNSUPPORTED, "dimension must be in [1, 4]");
    if (desc->order < 0 || desc->order > INTP_GPU_MAX_ORDER)
        return fail(INTP_ERR_UNSUPPORTED, "order must be in [0, 7]");
    if (desc->precision != INTP_PRECISION_FP64 && desc->precision != INTP_PRECISION_MIXED)
        return fail(INTP_ERR_INVALID_ARGUMENT, "unknown precision");
    if (desc->refine_steps < -1 || desc->refine_steps > 4)
        return fail(INTP_ERR_INVALID_ARGUMENT, "refine_steps must be in [-1, 4]");
    if (desc->channels < 0 || desc->channels > INTP_GPU_MAX_CHANNELS)
        return fail(INTP_ERR_INVALID_ARGUMENT, "channels must be in [0, 64]");
    TableSpec spec;
    spec.dim = desc->dim;
    spec.order = desc->order;
    for (int d = 0; d < desc->dim; ++d) {
        spec.periodic[d] = desc->periodic[d] != 0;
        spec.size[d] = desc->size[d];
        spec.lo[d] = desc->range_lo[d];
        spec.hi[d] = desc->range_hi[d];
        spec.coords[d] = desc->coords[d];
    }
    intp_table* t = new (std::nothrow) intp_table();
    if (!t) return fail(INTP_ERR_OUT_OF_MEMORY, "out of host memory");
    std::string err;
    try {
        err = build_model(spec, t->model);
    } catch (const std::bad_alloc&) {
        delete t;
        return fail(INTP_ERR_OUT_OF_MEMORY, "out of host memory");
    }
    if (!err.empty()) {
        delete t;
        return fail(INTP_ERR_INVALID_ARGUMENT, err);
    }
    t->precision = desc->precision;
    t->refine_steps = desc->refine_steps;
    t->channels = desc->channels > 1 ? desc->channels : 1;
    t->stream_ordered = stream_ordered;
    t->alloc_stream = stream;
    for (int d = 0; d < desc->dim; ++d) t->lo_user[d] = desc->range_lo[d];
    cudaGetDevice(&t->device);
    intp_status st = upload_table(t);
    if (st != INTP_OK) {
        delete t;
        return st;
    }
    *out = t;
    return INTP_OK;
}

size_t table_device_bytes(const intp_table* t) {
    return t->arena_bytes + static_cast<size_t>(t->values()) * (t->elem() + (t->ctrl_lo ? sizeof(float) : 0)) +
           t->scratch_bytes;
}

size_t table_build_scratch_bytes(const intp_table_desc* desc) {
    int64_t total = desc->channels > 1 ? desc->channels : 1;
    for (int d = 0; d < desc->dim && d < INTP_GPU_MAX_DIM; ++d) total *= desc->size[d];
    // values staging (FP64) plus, in the mixed form, the double-word solve's
    // working array (every channel)
    size_t b = static_cast<size_t>(total) * 8;
    if (desc->precision == INTP_PRECISION_MIXED) b += static_cast<size_t>(total) * sizeof(DW);
    return b;
}

void table_release_scratch(intp_table* t) {
    t->dfree(t->scratch);
    t->scratch = nullptr;
    t->scratch_bytes = 0;
}

int64_t table_values(const intp_table* t) { return t->values(); }

void pack_table(const TableModel& m, Arena& ar, PackedTable& pt) {
    const int O = m.order;
    for (int d = 0; d < m.dim; ++d) {
        const AxisModel& ax = m.axis[d];
        const std::vector<double>& t0 = ax.knots;
        const int64_t nk = static_cast<int64_t>(t0.size());
        std::vector<long long> keys(nk);
        std::vector<double> rinv(static_cast<size_t>(nk * std::max(O, 1)), 0.0);
        std::vector<float> kdf(static_cast<size_t>(nk * (2 * O + 2)), 0.0f), khi(nk), klo(nk);
        for (int64_t a = 0; a < nk; ++a) {
            unsigned long long b;
            std::memcpy(&b, &t0[a], 8);
            keys[a] = knot_key_bits(b);
            for (int s = 1; s <= O; ++s)
                if (a + s < nk && t0[a + s] != t0[a]) rinv[a * O + (s - 1)] = 1.0 / (t0[a + s] - t0[a]);
            for (int j = -O; j <= O + 1; ++j)
                if (a + j >= 0 && a + j < nk) kdf[a * (2 * O + 2) + (j + O)] = static_cast<float>(t0[a + j] - t0[a]);
            const uint32_t hb = split_hi_bits(b);
            float hf;
            std::memcpy(&hf, &hb, 4);
            khi[a] = hf;
            klo[a] = static_cast<float>(t0[a] - static_cast<double>(hf));
        }
        PackedTable::Axis& o = pt.ax[d];
        o.knots = ar.put(t0);
        o.keys = ar.put(keys);
        o.rinv = ar.put(rinv);
        o.rinvf = ar.put(to_f32(rinv));
        o.kdf = ar.put(kdf);
        o.khi = ar.put(khi);
        o.klo = ar.put(klo);
        const LineFactor& f = ax.factor;
        o.lower = ar.put(f.lower);
        o.upper = ar.put(f.upper);
        o.dinv = ar.put(f.dinv);
        o.bottom = ar.put(f.bottom);
        o.right = ar.put(f.right);
        o.lowerf = ar.put(to_f32(f.lower));
        o.upperf = ar.put(to_f32(f.upper));
        o.dinvf = ar.put(to_f32(f.dinv));
        o.bottomf = ar.put(to_f32(f.bottom));
        o.rightf = ar.put(to_f32(f.right));
        o.lowerw = ar.put(to_dw(f.lower));
        o.upperw = ar.put(to_dw(f.upper));
        o.dinvw = ar.put(to_dw(f.dinv));
        o.bottomw = ar.put(to_dw(f.bottom));
        o.rightw = ar.put(to_dw(f.right));
    }
}

void bind_table(const TableModel& m, const double* lo_user, const PackedTable& pt, const unsigned char* base,
                TableDev& dv, AxisFactorDev* fac) {
    const int O = m.order;
    dv.dim = m.dim;
    dv.order = O;
    dv.channels = 1;
    dv.chan_stride = m.total;
    int64_t stride = 1;
    for (int d = m.dim - 1; d >= 0; --d) {
        const AxisModel& ax = m.axis[d];
        AxisDev& a = dv.ax[d];
        const PackedTable::Axis& o = pt.ax[d];
        a.n = ax.n;
        a.nknots = static_cast<int64_t>(ax.knots.size());
        a.stride = stride;
        stride *= ax.n;
        a.periodic = ax.periodic ? 1 : 0;
        a.uniform = ax.uniform ? 1 : 0;
        a.lo = ax.range_lo;
        a.hi = ax.range_hi;
        a.period = ax.range_hi - ax.range_lo;
        a.ncells = a.nknots - 2 * O - 1;  // spans O .. nknots-O-2
        a.int_lo = 1;
        a.int_hi = 0;
        if (ax.uniform) {
            const int64_t extra = ax.periodic ? 2 * O + (1 - O % 2) : O + 1;
            a.hint_x0 = static_cast<float>(lo_user[d]);
            a.hint_inv_dx = static_cast<float>(1.0 / ax.dx);
            a.hint_off = static_cast<float>(0.5 * static_cast<double>(extra));
            a.inv_dxf = static_cast<float>(1.0 / ax.dx);
            // the basis at span c reads knots c-O+1 .. c+O; on a periodic axis
            // all knots are uniform, on a non-periodic one knots O+1 ..
            // nknots-O-2 are (the ends are clamped)
            if (ax.periodic) {
                a.int_lo = O;
                a.int_hi = a.nknots - O - 2;
            } else {
                a.int_lo = 2 * O;
                a.int_hi = a.nknots - 2 * O - 2;
            }
        }
        a.knots = reinterpret_cast<const double*>(base + o.knots);
        a.keys = reinterpret_cast<const long long*>(base + o.keys);
        a.rinv = reinterpret_cast<const double*>(base + o.rinv);
        a.rinvf = reinterpret_cast<const float*>(base + o.rinvf);
        a.kdf = reinterpret_cast<const float*>(base + o.kdf);
        a.khi = reinterpret_cast<const float*>(base + o.khi);
        a.klo = reinterpret_cast<const float*>(base + o.klo);
        AxisFactorDev& fd = fac[d];
        fd.lower = reinterpret_cast<const double*>(base + o.lower);
        fd.upper = reinterpret_cast<const double*>(base + o.upper);
        fd.dinv = reinterpret_cast<const double*>(base + o.dinv);
        fd.bottom = reinterpret_cast<const double*>(base + o.bottom);
        fd.right = reinterpret_cast<const double*>(base + o.right);
        fd.lowerf = reinterpret_cast<const float*>(base + o.lowerf);
        fd.upperf = reinterpret_cast<const float*>(base + o.upperf);
        fd.dinvf = reinterpret_cast<const float*>(base + o.dinvf);
        fd.bottomf = reinterpret_cast<const float*>(base + o.bottomf);
        fd.rightf = reinterpret_cast<const float*>(base + o.rightf);
        fd.lowerw = reinterpret_cast<const DW*>(base + o.lowerw);
        fd.upperw = reinterpret_cast<const DW*>(base + o.upperw);
        fd.dinvw = reinterpret_cast<const DW*>(base + o.dinvw);
        fd.bottomw = reinterpret_cast<const DW*>(base + o.bottomw);
        fd.rightw = reinterpret_cast<const DW*>(base + o.rightw);
        fd.clo = ax.factor.const_lo;
        fd.chi = ax.factor.const_hi;
        fd.clo32 = ax.factor.const_lo32;
        fd.chi32 = ax.factor.const_hi32;
        fd.zside = ax.factor.zside;
        fd.zside32 = ax.factor.zside32;
    }
}

void note_launch(int count) { g_launches.fetch_add(static_cast<unsigned long long>(count)); }
}  // namespace intp_gb300

extern "C" {

const char* intp_last_error(void) { return g_last_error.c_str(); }

uint64_t intp_launch_count(void) { return g_launches.load(); }

intp_status intp_table_create(const intp_table_desc* desc, intp_table** out) {
    return create_table(desc, false, nullptr, out);
}

intp_status intp_table_destroy(intp_table* table) {
    delete table;
    return INTP_OK;
}

intp_status intp_table_interpolate(intp_table* t, const double* values, int32_t values_on_device,
                                   void* stream) {
    if (!t || !values) return fail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t N = t->values();
    if (values_on_device) return run_interpolate(t, values, s);
    // host values: stage them on the device first
    void* stage = nullptr;
    INTP_CUDA(cudaMallocAsync(&stage, static_cast<size_t>(N) * 8, s), "cudaMallocAsync(values)");
    cudaError_t e = cudaMemcpyAsync(stage, values, static_cast<size_t>(N) * 8, cudaMemcpyHostToDevice, s);
    intp_status st = e == cudaSuccess ? run_interpolate(t, static_cast<double*>(stage), s)
                                      : cuda_fail(e, "cudaMemcpyAsync(values)");
    cudaFreeAsync(stage, s);
    return st;
}

// Control points cross the boundary as prod(size) x C doubles, channel
// fastest (the reference's plain mesh of T values); on the device each
// channel's mesh is contiguous.
intp_status intp_table_set_control_points(intp_table* t, const double* ctrl) {
    if (!t || !ctrl) return fail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    const int64_t P = t->model.total, C = t->channels, N = P * C;
    std::vector<double> v(static_cast<size_t>(N));
    for (int64_t i = 0; i < P; ++i)
        for (int64_t c = 0; c < C; ++c) v[c * P + i] = ctrl[i * C + c];
    if (t->mixed()) {
        // FP32 rounding, and its remainder where the table keeps one
        std::vector<float> f(static_cast<size_t>(N)), r(t->ctrl_lo ? static_cast<size_t>(N) : 0);
        for (int64_t i = 0; i < N; ++i) {
            f[i] = static_cast<float>(v[i]);
            if (t->ctrl_lo) r[i] = static_cast<float>(v[i] - static_cast<double>(f[i]));
        }
        INTP_CUDA(cudaMemcpy(t->ctrl, f.data(), N * 4, cudaMemcpyHostToDevice), "cudaMemcpy(ctrl)");
        if (t->ctrl_lo)
            INTP_CUDA(cudaMemcpy(t->ctrl_lo, r.data(), N * 4, cudaMemcpyHostToDevice), "cudaMemcpy(ctrl)");
    } else {
        INTP_CUDA(cudaMemcpy(t->ctrl, v.data(), N * 8, cudaMemcpyHostToDevice), "cudaMemcpy(ctrl)");
    }
    t->has_ctrl = true;
    return INTP_OK;
}

intp_status intp_table_get_control_points(const intp_table* t, double* out) {
    if (!t || !out) return fail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    if (!t->has_ctrl) return fail(INTP_ERR_STATE, "table has no control points yet");
    const int64_t P = t->model.total, C = t->channels, N = P * C;
    INTP_CUDA(cudaDeviceSynchronize(), "synchronize");
    std::vector<double> v(static_cast<size_t>(N));
    if (t->mixed()) {
        std::vector<float> f(static_cast<size_t>(N)), r(t->ctrl_lo ? static_cast<size_t>(N) : 0);
        INTP_CUDA(cudaMemcpy(f.data(), t->ctrl, N * 4, cudaMemcpyDeviceToHost), "cudaMemcpy(ctrl)");
        if (t->ctrl_lo)
            INTP_CUDA(cudaMemcpy(r.data(), t->ctrl_lo, N * 4, cudaMemcpyDeviceToHost), "cudaMemcpy(ctrl)");
        for (int64_t i = 0; i < N; ++i)
            v[i] = static_cast<double>(f[i]) + (t->ctrl_lo ? static_cast<double>(r[i]) : 0.0);
    } else {
        INTP_CUDA(cudaMemcpy(v.data(), t->ctrl, N * 8, cudaMemcpyDeviceToHost), "cudaMemcpy(ctrl)");
    }
    for (int64_t i = 0; i < P; ++i)
        for (int64_t c = 0; c < C; ++c) out[i * C + c] = v[c * P + i];
    return INTP_OK;
}

intp_status intp_table_axis_info(const intp_table* t, int32_t axis, int64_t* nknots, double* lo,
                                 double* hi, int32_t* periodic, int32_t* uniform) {
    if (!t) return fail(INTP_ERR_INVALID_ARGUMENT, "null table");
    if (axis < 0 || axis >= t->model.dim) return fail(INTP_ERR_INVALID_ARGUMENT, "axis out of range");
    const AxisModel& ax = t->model.axis[axis];
    if (nknots) *nknots = static_cast<int64_t>(ax.knots.size());
    if (lo) *lo = ax.range_lo;
    if (hi) *hi = ax.range_hi;
    if (periodic) *periodic = ax.periodic ? 1 : 0;
    if (uniform) *uniform = ax.uniform ? 1 : 0;
    return INTP_OK;
}

intp_status intp_table_knots(const intp_table* t, int32_t axis, double* out) {
    if (!t || !out) return fail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    if (axis < 0 || axis >= t->model.dim) return fail(INTP_ERR_INVALID_ARGUMENT, "axis out of range");
    const AxisModel& ax = t->model.axis[axis];
    std::memcpy(out, ax.knots.data(), ax.knots.size() * sizeof(double));
    return INTP_OK;
}

intp_status intp_eval(const intp_table* t, const double* coords, int64_t npts, const int32_t* derivs,
                      int32_t nderiv, void* out, int32_t out_dtype, void* stream) {
    if (!t) return fail(INTP_ERR_INVALID_ARGUMENT, "null table");
    if (npts < 0) return fail(INTP_ERR_INVALID_ARGUMENT, "npts must be >= 0");
    if (npts > 0 && (!coords || !out)) return fail(INTP_ERR_INVALID_ARGUMENT, "null buffer");
    if (!t->has_ctrl) return fail(INTP_ERR_STATE, "table has no control points yet");
    if (out_dtype != INTP_F64 && out_dtype != INTP_F32)
        return fail(INTP_ERR_INVALID_ARGUMENT, "unknown output dtype");
    DerivPlan plan;
    std::string err;
    if (!make_plan(t, derivs, nderiv, plan, err)) return fail(INTP_ERR_INVALID_ARGUMENT, err);
    const int mode = eval_mode();
    // binned needs the per-bucket counters to fit in shared memory; plans
    // that take the precise contraction read the control points' remainders
    // per query and evaluate with the direct kernel
    const bool binned = t->mixed() && t->model.dim <= 3 && t->bins.smem_buckets > 0 && !plan.precise &&
                        (mode == 2 || (mode == 0 && npts >= kBinnedMinPoints));
    if (binned) {
        retain_pool_memory();
        INTP_CUDA(run_binned_eval(t->dev, t->bins, t->has_tile_map ? t->tile_map : nullptr, coords, npts, plan, out,
                                  out_dtype == INTP_F32, eval_chunk(), static_cast<cudaStream_t>(stream)),
                  "binned evaluation");
        return INTP_OK;
    }
    INTP_CUDA(launch_eval_direct(t->dev, t->mixed(), coords, npts, plan, out, out_dtype == INTP_F32,
                                 static_cast<cudaStream_t>(stream)),
              "evaluation kernel");
    return INTP_OK;
}

intp_status intp_eval_host(const intp_table* t, const double* coords, int64_t npts,
                           const int32_t* derivs, int32_t nderiv, void* out, int32_t out_dtype,
                           void* stream) {
    if (!t) return fail(INTP_ERR_INVALID_ARGUMENT, "null table");
    if (npts < 0) return fail(INTP_ERR_INVALID_ARGUMENT, "npts must be >= 0");
    if (npts == 0) return INTP_OK;
    if (!coords || !out) return fail(INTP_ERR_INVALID_ARGUMENT, "null buffer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int D = t->model.dim;
    const int K = (derivs ? nderiv : 1) * t->channels;  // output values per point
    const size_t osz = out_dtype == INTP_F32 ? 4 : 8;
    // pipeline chunks: the copies of one chunk overlap the evaluation of the
    // next; the largest stays within the sort's own chunk
    const int64_t chunk = std::min<int64_t>(eval_chunk(), kHostPipelineChunk);
    if (npts <= std::min(chunk, kHostHeadChunk)) {
        const size_t cb = static_cast<size_t>(npts) * D * 8;
        const size_t ob = static_cast<size_t>(npts) * K * osz;
        void *dc = nullptr, *dout = nullptr;
        INTP_CUDA(cudaMallocAsync(&dc, cb, s), "cudaMallocAsync(coords)");
        cudaError_t e = cudaMallocAsync(&dout, ob, s);
        if (e != cudaSuccess) {
            cudaFreeAsync(dc, s);
            return cuda_fail(e, "cudaMallocAsync(out)");
        }
        intp_status st = INTP_OK;
        e = cudaMemcpyAsync(dc, coords, cb, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaMemcpyAsync(coords)");
        if (st == INTP_OK) st = intp_eval(t, static_cast<double*>(dc), npts, derivs, nderiv, dout, out_dtype, stream);
        if (st == INTP_OK) {
            e = cudaMemcpyAsync(out, dout, ob, cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) st = cuda_fail(e, "cudaMemcpyAsync(out)");
        }
        cudaFreeAsync(dc, s);
        cudaFreeAsync(dout, s);
        e = cudaStreamSynchronize(s);
        if (st == INTP_OK && e != cudaSuccess) st = cuda_fail(e, "cudaStreamSynchronize");
        return st;
    }
    // Several chunks, kHostBuffers device buffers of each kind: the copy of
    // chunk i+1 in and of chunk i-1 out overlap the evaluation of chunk i.
    // The copy-in stream allocates its own buffers and does not wait for work
    // queued earlier on the caller's stream, so the coordinates stream in
    // while that work (typically the table's solve) runs; every evaluation
    // still runs after it. The copy-in bounds the pipeline (the link moves
    // fewer points per second than the evaluation), so chunks grow from
    // kHostHeadChunk (the first evaluation starts early) and then never take
    // more than half of the points left: the last chunks shrink
    // geometrically down to the head chunk, and little evaluation and
    // copy-out remains after the last copy-in.
    constexpr int NB = kHostBuffers;
    cudaStream_t h2d = nullptr, d2h = nullptr;
    cudaEvent_t in_ready[NB] = {}, done[NB] = {}, freed[NB] = {};
    void* din[NB] = {};
    void* dout[NB] = {};
    const size_t cb = static_cast<size_t>(chunk) * D * 8, ob = static_cast<size_t>(chunk) * K * osz;
    cudaError_t e = cudaStreamCreateWithFlags(&h2d, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&d2h, cudaStreamNonBlocking);
    for (int j = 0; j < NB && e == cudaSuccess; ++j) {
        e = cudaEventCreateWithFlags(&in_ready[j], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done[j], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&freed[j], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMallocAsync(&din[j], cb, h2d);
        if (e == cudaSuccess) e = cudaMallocAsync(&dout[j], ob, s);
    }
    intp_status st = e == cudaSuccess ? INTP_OK : cuda_fail(e, "pipelined evaluation set-up");
    int64_t i = 0;
    int64_t cur = std::min(chunk, kHostHeadChunk);
    for (int64_t p0 = 0; p0 < npts && st == INTP_OK; ++i) {
        const int j = static_cast<int>(i % NB);
        const int64_t rem = npts - p0;
        const int64_t head = std::min(chunk, kHostHeadChunk);
        // (what is left after a chunk is never below the head chunk, so every
        // chunk of a batch takes the path one device call on it would take)
        const int64_t n =
            std::min(chunk, rem <= 2 * head ? rem : std::min(cur, std::max(head, (rem + 1) / 2)));
        cur = std::min(cur * 2, chunk);
        // buffer j's previous chunk: evaluated (input free) and copied out (output free)
        if (i >= NB) e = cudaStreamWaitEvent(h2d, done[j], 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(din[j], coords + p0 * D, static_cast<size_t>(n) * D * 8, cudaMemcpyHostToDevice, h2d);
        if (e == cudaSuccess) e = cudaEventRecord(in_ready[j], h2d);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, in_ready[j], 0);
        if (e == cudaSuccess && i >= NB) e = cudaStreamWaitEvent(s, freed[j], 0);
        if (e != cudaSuccess) {
            st = cuda_fail(e, "pipelined evaluation (copy in)");
            break;
        }
        st = intp_eval(t, static_cast<double*>(din[j]), n, derivs, nderiv, dout[j], out_dtype, stream);
        if (st != INTP_OK) break;
        e = cudaEventRecord(done[j], s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(d2h, done[j], 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(static_cast<unsigned char*>(out) + static_cast<size_t>(p0) * K * osz, dout[j],
                                static_cast<size_t>(n) * K * osz, cudaMemcpyDeviceToHost, d2h);
        if (e == cudaSuccess) e = cudaEventRecord(freed[j], d2h);
        if (e != cudaSuccess) st = cuda_fail(e, "pipelined evaluation (copy out)");
        p0 += n;
    }
    // the caller's stream resumes after both copy streams; then release
    for (cudaStream_t cs : {h2d, d2h}) {
        cudaEvent_t fin = nullptr;
        if (cs && cudaEventCreateWithFlags(&fin, cudaEventDisableTiming) == cudaSuccess) {
            cudaEventRecord(fin, cs);
            cudaStreamWaitEvent(s, fin, 0);
            cudaEventDestroy(fin);
        }
    }
    for (int j = 0; j < NB; ++j) {
        if (din[j]) cudaFreeAsync(din[j], s);
        if (dout[j]) cudaFreeAsync(dout[j], s);
    }
    e = cudaStreamSynchronize(s);
    if (st == INTP_OK && e != cudaSuccess) st = cuda_fail(e, "cudaStreamSynchronize");
    if (h2d) cudaStreamSynchronize(h2d);
    if (d2h) cudaStreamSynchronize(d2h);
    for (int j = 0; j < NB; ++j) {
        if (in_ready[j]) cudaEventDestroy(in_ready[j]);
        if (done[j]) cudaEventDestroy(done[j]);
        if (freed[j]) cudaEventDestroy(freed[j]);
    }
    if (h2d) cudaStreamDestroy(h2d);
    if (d2h) cudaStreamDestroy(d2h);
    return st;
}

intp_status intp_check_range(const intp_table* t, const double* coords, int64_t npts, int64_t* first_bad,
                             void* stream) {
    if (!t || !first_bad) return fail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    *first_bad = -1;
    if (npts <= 0) return INTP_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned long long* d = nullptr;
    INTP_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&d), 8, s), "cudaMallocAsync");
    const unsigned long long init = ~0ULL;
    intp_status st = INTP_OK;
    cudaError_t e = cudaMemcpyAsync(d, &init, 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_range_check(t->dev, coords, npts, d, s);
    unsigned long long h = ~0ULL;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_fail(e, "range check");
    if (st == INTP_OK && h != ~0ULL) *first_bad = static_cast<int64_t>(h);
    return st;
}

intp_status intp_locate(const intp_table* t, const double* coords, int64_t npts, int64_t* cells,
                        double* wrapped, void* stream) {
    if (!t || (npts > 0 && (!coords || !cells))) return fail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    INTP_CUDA(launch_locate(t->dev, coords, npts, cells, wrapped, static_cast<cudaStream_t>(stream)),
              "locate kernel");
    return INTP_OK;
}

intp_status intp_proxy_create(const intp_table* t, const double* coords, int64_t npts, void* stream,
                              intp_proxy** out) {
    if (!t || !out || (npts > 0 && !coords)) return fail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (npts < 0) return fail(INTP_ERR_INVALID_ARGUMENT, "npts must be >= 0");
    if (t->model.dim > 3 || t->channels != 1)
        return fail(INTP_ERR_UNSUPPORTED, "evaluation proxies take scalar tables of dimension 1..3");
    const int D = t->model.dim, W = t->model.order + 1;
    const size_t rb = t->mixed() ? 4 : 8;
    const size_t n = static_cast<size_t>(npts);
    auto up = [](size_t v) { return (v + 255) & ~size_t(255); };
    const size_t b_c = up(n * D * 8), b_x = up(n * D * rb), b_w = up(n * D * W * rb);
    intp_proxy* p = new (std::nothrow) intp_proxy();
    if (!p) return fail(INTP_ERR_OUT_OF_MEMORY, "out of host memory");
    p->device = t->device;
    p->precision = t->precision;
    p->dim = D;
    p->order = t->model.order;
    for (int d = 0; d < D; ++d) {
        p->periodic[d] = t->model.axis[d].periodic;
        p->knots[d] = t->model.axis[d].knots;
    }
    p->npts = npts;
    if (npts > 0) {
        const cudaError_t e = cudaMalloc(&p->mem, b_c + b_x + b_w);
        if (e != cudaSuccess) {
            delete p;
            return cuda_fail(e, "cudaMalloc(proxy)");
        }
        unsigned char* m = static_cast<unsigned char*>(p->mem);
        p->cells = reinterpret_cast<int64_t*>(m);
        p->xr = m + b_c;
        p->base = m + b_c + b_x;
        const cudaError_t e2 = launch_proxy_build(t->dev, t->mixed(), coords, npts, p->cells, p->xr, p->base,
                                                  static_cast<cudaStream_t>(stream));
        if (e2 != cudaSuccess) {
            delete p;
            return cuda_fail(e2, "proxy kernel");
        }
    }
    *out = p;
    return INTP_OK;
}

intp_status intp_proxy_destroy(intp_proxy* p) {
    delete p;
    return INTP_OK;
}

intp_status intp_proxy_eval(const intp_proxy* p, const intp_table* const* tables, int32_t ntables, void* out,
                            int32_t out_dtype, void* stream) {
    if (!p || (ntables > 0 && !tables) || (p->npts > 0 && ntables > 0 && !out))
        return fail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    if (ntables < 0) return fail(INTP_ERR_INVALID_ARGUMENT, "ntables must be >= 0");
    if (out_dtype != INTP_F32 && out_dtype != INTP_F64) return fail(INTP_ERR_INVALID_ARGUMENT, "unknown output dtype");
    if (ntables == 0 || p->npts == 0) return INTP_OK;
    std::vector<TableDev> devs(static_cast<size_t>(ntables));
    for (int32_t j = 0; j < ntables; ++j) {
        const intp_table* t = tables[j];
        if (!t) return fail(INTP_ERR_INVALID_ARGUMENT, "null table");
        if (!t->has_ctrl) return fail(INTP_ERR_STATE, "table has no control points yet");
        bool same = t->model.dim == p->dim && t->model.order == p->order && t->precision == p->precision &&
                    t->channels == 1 && t->device == p->device;
        for (int d = 0; same && d < p->dim; ++d)
            same = t->model.axis[d].periodic == p->periodic[d] && t->model.axis[d].knots == p->knots[d];
        if (!same) return fail(INTP_ERR_INVALID_ARGUMENT, "table does not share the proxy's knots");
        devs[static_cast<size_t>(j)] = t->dev;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DerivPlan plan{};
    std::string err;
    if (!make_plan(tables[0], nullptr, 0, plan, err)) return fail(INTP_ERR_INVALID_ARGUMENT, err);
    TableDev* dd = nullptr;
    const size_t bytes = devs.size() * sizeof(TableDev);
    INTP_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&dd), bytes, s), "cudaMallocAsync(proxy tables)");
    cudaError_t e = cudaMemcpyAsync(dd, devs.data(), bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = launch_proxy_eval(dd, ntables, p->dim, p->order, p->precision == INTP_PRECISION_MIXED, p->npts,
                              p->cells, p->xr, p->base, plan, out, out_dtype == INTP_F32 ? 1 : 0, s);
    // the descriptors are read from pageable host memory by the copy: wait for
    // it before `devs` goes out of scope
    const cudaError_t e2 = cudaFreeAsync(dd, s);
    const cudaError_t e3 = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "proxy evaluation");
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaFreeAsync(proxy tables)");
    if (e3 != cudaSuccess) return cuda_fail(e3, "cudaStreamSynchronize");
    return INTP_OK;
}

intp_status intp_locate_binned(const intp_table* t, const double* coords, int64_t npts, int64_t* cells,
                               void* stream) {
    if (!t || (npts > 0 && (!coords || !cells))) return fail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    if (npts < 0) return fail(INTP_ERR_INVALID_ARGUMENT, "npts must be >= 0");
    if (!(t->mixed() && t->model.dim <= 3 && t->channels == 1 && t->bins.smem_buckets > 0))
        return fail(INTP_ERR_UNSUPPORTED, "the table does not take the binned evaluation path");
    INTP_CUDA(binned_span_readout(t->dev, t->bins, coords, npts, cells, static_cast<cudaStream_t>(stream)),
              "binned span read-out");
    return INTP_OK;
}

intp_status intp_debug_set_wait_limit(uint32_t probes) {
    INTP_CUDA(set_wait_probes_bin_d3(probes), "cudaMemcpyToSymbol(wait probes)");
    INTP_CUDA(set_wait_probes_bin_d12(probes), "cudaMemcpyToSymbol(wait probes)");
    return INTP_OK;
}

intp_status intp_debug_set_segment_warmup(int32_t rows) {
    if (rows < -1) return fail(INTP_ERR_INVALID_ARGUMENT, "rows must be >= -1");
    INTP_CUDA(set_warm_cap_solve(rows), "cudaMemcpyToSymbol(warm-up cap)");
    INTP_CUDA(set_warm_cap_batch(rows), "cudaMemcpyToSymbol(warm-up cap)");
    return INTP_OK;
}

intp_status intp_debug_fail_allocations(int32_t count) {
    if (count < 0) return fail(INTP_ERR_INVALID_ARGUMENT, "count must be >= 0");
    g_fail_allocs.store(count);
    return INTP_OK;
}

intp_status intp_stream_synchronize(void* stream) {
    INTP_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "cudaStreamSynchronize");
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int err = take_device_error(s) | take_device_error_bin_d12(s) | take_device_error_bin_d3(s);
    if (err != 0)
        return fail(INTP_ERR_TIMEOUT, "a kernel's bounded wait for an asynchronous copy ran out");
    return INTP_OK;
}

intp_status intp_host_alloc(size_t bytes, void** ptr) {
    if (!ptr) return fail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    *ptr = nullptr;
    if (bytes == 0) return INTP_OK;
    INTP_CUDA(cudaHostAlloc(ptr, bytes, cudaHostAllocPortable), "cudaHostAlloc");
    return INTP_OK;
}

intp_status intp_host_free(void* ptr) {
    if (ptr) INTP_CUDA(cudaFreeHost(ptr), "cudaFreeHost");
    return INTP_OK;
}

intp_status intp_bandlu_create(int64_t n, int32_t p, int32_t q, int32_t cyclic, const double* band,
                               const double* right, const double* bottom, intp_bandlu** out) {
    if (!out || !band) return fail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (p != q || p < 0 || p > (cyclic ? 3 : 6))
        return fail(INTP_ERR_UNSUPPORTED, "band widths must satisfy p == q <= 6 (<= 3 cyclic)");
    if (n < 2 * p + 1) return fail(INTP_ERR_INVALID_ARGUMENT, "matrix too small for its bands");
    if (cyclic && (!right || !bottom) && p > 0)
        return fail(INTP_ERR_INVALID_ARGUMENT, "cyclic matrices need the side bands");
    BandStore m;
    m.reset(n, p, q, cyclic != 0);
    std::memcpy(m.band.data(), band, static_cast<size_t>(n * (1 + p + q)) * 8);
    if (cyclic && p > 0) {
        std::memcpy(m.right.data(), right, static_cast<size_t>((n - q - 1) * p) * 8);
        std::memcpy(m.bottom.data(), bottom, static_cast<size_t>((n - p - 1) * q) * 8);
    }
    m.factorize();
    intp_bandlu* lu = new (std::nothrow) intp_bandlu();
    if (!lu) return fail(INTP_ERR_OUT_OF_MEMORY, "out of host memory");
    lu->f = line_factor_from(m);
    Arena ar;
    const size_t ol = ar.put(lu->f.lower), ou = ar.put(lu->f.upper), od = ar.put(lu->f.dinv),
                 ob = ar.put(lu->f.bottom), orr = ar.put(lu->f.right);
    cudaError_t e = cudaMalloc(&lu->arena, ar.host.size());
    if (e == cudaSuccess) e = cudaMemcpy(lu->arena, ar.host.data(), ar.host.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        delete lu;
        return cuda_fail(e, "band LU upload");
    }
    unsigned char* b = static_cast<unsigned char*>(lu->arena);
    lu->lower = reinterpret_cast<const double*>(b + ol);
    lu->upper = reinterpret_cast<const double*>(b + ou);
    lu->dinv = reinterpret_cast<const double*>(b + od);
    lu->bottom = reinterpret_cast<const double*>(b + ob);
    lu->right = reinterpret_cast<const double*>(b + orr);
    *out = lu;
    return INTP_OK;
}

intp_status intp_bandlu_solve(const intp_bandlu* lu, double* x, int64_t outer, int64_t inner,
                              void* stream) {
    if (!lu || !x) return fail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    if (outer < 1 || inner < 1) return fail(INTP_ERR_INVALID_ARGUMENT, "empty tensor");
    INTP_CUDA(launch_line_solve_f64(x, lu->f.n, inner, outer * inner, lu->f.p, lu->f.q, lu->f.cyclic,
                                    lu->lower, lu->upper, lu->dinv, lu->bottom, lu->right,
                                    static_cast<cudaStream_t>(stream)),
              "band solve");
    return INTP_OK;
}

intp_status intp_bandlu_destroy(intp_bandlu* lu) {
    delete lu;
    return INTP_OK;
}

intp_status intp_eval_noalloc(const intp_table* t, const double* coords, int64_t npts, const int32_t* derivs,
                              int32_t nderiv, void* out, int32_t out_dtype, void* stream) {
    if (!t) return fail(INTP_ERR_INVALID_ARGUMENT, "null table");
    if (npts < 0) return fail(INTP_ERR_INVALID_ARGUMENT, "npts must be >= 0");
    if (npts > 0 && (!coords || !out)) return fail(INTP_ERR_INVALID_ARGUMENT, "null buffer");
    if (!t->has_ctrl) return fail(INTP_ERR_STATE, "table has no control points yet");
    if (out_dtype != INTP_F64 && out_dtype != INTP_F32)
        return fail(INTP_ERR_INVALID_ARGUMENT, "unknown output dtype");
    DerivPlan plan;
    std::string err;
    if (!make_plan(t, derivs, nderiv, plan, err)) return fail(INTP_ERR_INVALID_ARGUMENT, err);
    int dev = -1;
    INTP_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev != t->device) return fail(INTP_ERR_INVALID_ARGUMENT, "make the table's device current first");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool out_f32 = out_dtype == INTP_F32;
    // the array's address first, whatever the table: any first call on a
    // device (npts = 0 included) does the set-up
    void* base = nullptr;
    const intp_status st = noalloc_scratch_address(dev, &base);
    if (st != INTP_OK) return st;
    const bool bins = t->mixed() && t->model.dim <= 3 && t->channels == 1 && t->bins.smem_buckets > 0;
    // carve the fixed area: per-(bucket, CTA) counts and offsets, scan tile
    // sums, then as many query records as fit
    const int D = t->model.dim;
    const BinGeom& g = t->bins;
    const int64_t m = bins ? g.nbuckets * kNoAllocSortBlocks : 0;
    auto up = [](size_t v) { return (v + 255) & ~size_t(255); };
    const size_t fixed = up(static_cast<size_t>(m) * 4) * 2 + up(static_cast<size_t>((m + 4095) / 4096) * 4);
    // per query: its record (in bucket order)
    const size_t per_rec = static_cast<size_t>(4 * bin_record_words(D));
    if (bins && fixed + 1024 * per_rec + 512 > kNoAllocScratchBytes)
        return fail(INTP_ERR_INVALID_ARGUMENT,
                    "table has too many buckets (" + std::to_string(g.nbuckets) +
                        ") for the 8 MiB scratch of the allocation-free evaluation; use intp_eval");
    if (npts == 0) return INTP_OK;
    if (!bins || npts < kBinnedMinPoints || plan.precise) {
        // the direct kernel needs no scratch: tables the binned path does not
        // take, and batches too small to be worth binning (as intp_eval)
        INTP_CUDA(launch_eval_direct(t->dev, t->mixed(), coords, npts, plan, out, out_f32, s), "evaluation kernel");
        return INTP_OK;
    }
    int64_t cap = static_cast<int64_t>((kNoAllocScratchBytes - fixed - 512) / per_rec);
    cap &= ~int64_t{63};
    unsigned char* p = static_cast<unsigned char*>(base);
    uint32_t* blkcount = reinterpret_cast<uint32_t*>(p);
    p += up(static_cast<size_t>(m) * 4);
    uint32_t* blkoffset = reinterpret_cast<uint32_t*>(p);
    p += up(static_cast<size_t>(m) * 4);
    uint32_t* tile_sum = reinterpret_cast<uint32_t*>(p);
    p += up(static_cast<size_t>((m + 4095) / 4096) * 4);
    uint32_t* rec = reinterpret_cast<uint32_t*>(p);
    // every word the kernels read is written earlier in the same chunk (counts
    // by the count kernel, offsets by the scan, records by the scatter), so
    // nothing in the area has to be cleared between calls
    int sms = 1;
    INTP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
    const size_t ob = out_f32 ? 4 : 8;
    for (int64_t p0 = 0; p0 < npts; p0 += cap) {
        const int64_t n = std::min(cap, npts - p0);
        int64_t slice = 0;
        INTP_CUDA(bin_sort_chunk(t->dev, g, coords + p0 * D, n, kNoAllocSortBlocks, blkcount, blkoffset, tile_sum,
                                 rec, &slice, s),
                  "binned sort");
        void* o = static_cast<unsigned char*>(out) + static_cast<size_t>(p0) * plan.k * ob;
        const CUtensorMap* tm = t->has_tile_map ? t->tile_map : nullptr;
        INTP_CUDA(D <= 2 ? launch_bin_eval_d12(t->dev, g, tm, blkoffset, kNoAllocSortBlocks, slice, rec, n, plan, o,
                                               out_f32, sms, s)
                         : launch_bin_eval_d3(t->dev, g, tm, blkoffset, kNoAllocSortBlocks, slice, rec, n, plan, o,
                                              out_f32, sms, s),
                  "binned evaluation");
    }
    return INTP_OK;
}

}  // extern "C"
