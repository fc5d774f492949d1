// Batched tables: thousands of independent interpolation tables of uneven
// size, order, periodicity and dimension (1..3), built and evaluated
// together.
//
// A batch packs the per-axis data of every table into one device arena and
// the control points of every table into one array (table i at element
// offset off[i]). The control-point solve of all tables runs as one launch
// per axis pass: pass j solves axis D_i - 1 - j of every table i that has
// one, as a work list of line groups (one warp per group of up to 32 lines),
// longest lines first. The arithmetic per line is solve_line_chunked, the same as the
// single-table solves, so a batched table gets the control points that
// intp_table_interpolate gives it, bit for bit. Mixed-precision batches
// solve each table in double-word arithmetic (R = DW, control points kept
// as FP32 pairs), or in FP32 for tables built with refine_steps = 0, as a
// single table is.
//
// Evaluation takes one list of query runs per (dimension, order) class and
// evaluates each run with the per-point code of the direct kernel
// (eval_point), so batched results equal intp_eval's direct path bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "batch.hpp"
#include "intp_gpu.h"
#include "launch.hpp"
#include "solve_line.cuh"
#include "spline_model.hpp"
#include "table_pack.hpp"

using namespace intp_gb300;

namespace {

constexpr int32_t kChunkElems = 8192;
constexpr int64_t kEvalRun = 2048;           // query points per evaluation CTA
// work counters of one build's persistent launches: a pass per axis, a
// launch per band class, and a mixed batch's FP32 and double-word solves
constexpr int kMaxLaunches = 2 * kBatchMaxDim * kBatchClasses;

intp_status bfail(intp_status s, const std::string& msg);

}  // namespace

struct intp_batch {
    int precision = INTP_PRECISION_MIXED;
    int device = 0;
    int64_t ntables = 0;
    std::vector<TableModel> models;
    std::vector<int64_t> off;      // ntables + 1 element offsets (every channel)
    std::vector<int> channels;     // values per mesh point of each table (vector-valued tables)
    // mixed: per table 0 (FP32 solve) or > 0 (double-word solve, control
    // points kept as ctrl + ctrl_lo); the largest and the smallest value
    std::vector<int> refine;
    int max_refine = 0, min_refine = 1 << 30;
    std::vector<TableDev> h_tables;
    void* arena = nullptr;         // per-axis data, descriptors, work lists
    void* ctrl = nullptr;
    float* ctrl_lo = nullptr;      // control-point remainders of refining tables (mixed)
    void* scratch = nullptr;       // refinement buffers
    size_t scratch_bytes = 0;
    TableDev* d_tables = nullptr;
    const AxisFactorDev* d_fac = nullptr;  // [ntables * kBatchMaxDim]
    const int64_t* d_off = nullptr;
    const int32_t* d_refine = nullptr;
    const ChunkItem* d_chunks = nullptr;
    int64_t nchunks = 0;
    // One axis pass: its work items in one list per band class, a launch
    // each, in the order of `order` (most values first).
    struct Pass {
        const SolveItem* items[kBatchClasses] = {};
        int64_t nitems[kBatchClasses] = {};
        int order[kBatchClasses] = {};
        int nclasses = 0;
    } pass[kBatchMaxDim];
    int npasses = 0;
    bool has_ctrl = false;
    intp_batch_schedule sched{0, 32, 32, 0, 0.0};
    void* work = nullptr;                // the schedule's work lists (device)
    uint64_t work_version = 0;           // bumped whenever the work lists are replaced
    unsigned int* counters = nullptr;    // work counters of the persistent passes (device)
    // The band classes of one pass run concurrently: class order[0] on the
    // caller's stream, the others on these streams, forked from and joined
    // back to the caller's stream by events (created on first need).
    cudaStream_t side[kBatchClasses - 1] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[kBatchClasses - 1] = {};
    int nside = 0;

    ~intp_batch() {
        for (int k = 0; k < nside; ++k) {
            cudaStreamDestroy(side[k]);
            cudaEventDestroy(join[k]);
        }
        if (fork) cudaEventDestroy(fork);
        if (work) cudaFree(work);
        if (counters) cudaFree(counters);
        if (arena) cudaFree(arena);
        if (ctrl) cudaFree(ctrl);
        if (ctrl_lo) cudaFree(ctrl_lo);
        if (scratch) cudaFree(scratch);
    }
    bool mixed() const { return precision == INTP_PRECISION_MIXED; }
    size_t elem() const { return mixed() ? sizeof(float) : sizeof(double); }
};

namespace {

intp_status bfail(intp_status s, const std::string& msg) {
    set_last_error(msg);
    return s;
}

intp_status bcuda(cudaError_t e, const char* what) {
    set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? INTP_ERR_OUT_OF_MEMORY : INTP_ERR_CUDA;
}

#define BATCH_CUDA(call, what)                           \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return bcuda(e_, what);   \
    } while (0)

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

}  // namespace

namespace intp_gb300 {
cudaError_t set_warm_cap_batch(int rows) {
    cudaError_t e = set_warm_cap_batch_f32(rows);
    if (e == cudaSuccess) e = set_warm_cap_batch_dw(rows);
    if (e == cudaSuccess) e = set_warm_cap_batch_f64(rows);
    return e;
}
}  // namespace intp_gb300

namespace {

// Element-wise passes over chunk items:
//  op 0: dst[shift(i)] = (R) src[i]; in a mixed batch, for the tables solved
//        in double-word arithmetic (refine > 0), the double-word split of
//        src[i] into w[shift(i)] instead (the single-table shift copy's)
//  op 1: (ctrl, ctrl_lo)[i] = (w[i].hi, w[i].lo)  (refine > 0 tables only)
// The periodic shift moves index i to (i + O/2) mod n along every periodic
// axis (InterpolationTemplate.hpp:451-462).
template <class R>
__global__ void __launch_bounds__(256) batch_elementwise_kernel(int op, const double* __restrict__ src,
                                                                R* __restrict__ dst, DW* __restrict__ w,
                                                                float* __restrict__ ctrl_lo,
                                                                const ChunkItem* __restrict__ chunks,
                                                                const TableDev* __restrict__ tables,
                                                                const int64_t* __restrict__ off,
                                                                const int32_t* __restrict__ refine) {
    const ChunkItem c = chunks[blockIdx.x];
    const bool dw = w && refine[c.table] > 0;
    if (op != 0 && !dw) return;
    const int64_t o0 = off[c.table];
    // each thread moves kU elements per step, their loads issued together
    constexpr int kU = 4;
    const int step = kU * blockDim.x;
    if (op == 0) {
        const TableDev& t = tables[c.table];
        // vector-valued tables: input element j is point j / C, channel
        // j % C (channel fastest); channel ch's mesh starts at ch * chan_stride
        const int C = t.channels;
        bool shifted = C > 1;
        for (int d = 0; d < t.dim; ++d) shifted = shifted || (t.ax[d].periodic && (t.order / 2) % t.ax[d].n != 0);
        for (int e0 = threadIdx.x; e0 < c.len; e0 += step) {
            double v[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int e = e0 + u * blockDim.x;
                v[u] = e < c.len ? src[o0 + c.start + e] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int e = e0 + u * blockDim.x;
                if (e >= c.len) break;
                // batched tables hold fewer than 2^31 values each: 32-bit
                // index math
                int o = static_cast<int>(c.start + e);
                if (shifted) {
                    const int pt = o / C, ch = o - pt * C;
                    int r = pt;
                    o = ch * static_cast<int>(t.chan_stride);
                    for (int d = t.dim - 1; d >= 0; --d) {
                        const AxisDev& a = t.ax[d];
                        const int na = static_cast<int>(a.n);
                        const int q = r / na;
                        int idx = r - q * na;
                        r = q;
                        if (a.periodic) {
                            idx += (t.order / 2) % na;
                            if (idx >= na) idx -= na;
                        }
                        o += idx * static_cast<int>(a.stride);
                    }
                }
                if (dw) {
                    float h, l;
                    split_double(v[u], h, l);
                    w[o0 + o] = DW(h, l);
                } else {
                    dst[o0 + o] = static_cast<R>(v[u]);
                }
            }
        }
    } else {
        float* x = reinterpret_cast<float*>(dst);
        for (int e0 = threadIdx.x; e0 < c.len; e0 += step) {
            DW v[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int e = e0 + u * blockDim.x;
                v[u] = e < c.len ? w[o0 + c.start + e] : DW(0.0f, 0.0f);
            }
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int e = e0 + u * blockDim.x;
                if (e >= c.len) break;
                x[o0 + c.start + e] = v[u].hi;
                ctrl_lo[o0 + c.start + e] = v[u].lo;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------

size_t up256(size_t v) { return (v + 255) & ~size_t(255); }

// Work lists of the axis passes under a schedule (lines per item on the
// contiguous and on the strided axes), one list per (pass, band class) at
// index pass * kBatchClasses + class, with the values each list covers, and
// the value chunks of the element-wise kernels.
void build_work(const intp_batch& b, const intp_batch_schedule& sc, std::vector<std::vector<SolveItem>>& passes,
                std::vector<int64_t>& values, std::vector<ChunkItem>& chunks) {
    passes.assign(static_cast<size_t>(kBatchMaxDim) * kBatchClasses, {});
    values.assign(passes.size(), 0);
    chunks.clear();
    for (int64_t i = 0; i < b.ntables; ++i) {
        const TableModel& m = b.models[i];
        const int C = b.channels[i];
        for (int j = 0; j < m.dim; ++j) {
            const int a = m.dim - 1 - j;
            const int64_t n = m.axis[a].n;
            const int64_t nlines = m.total / n;
            const bool contig = (a == m.dim - 1);
            const int64_t rows_max = contig ? sc.contig_rows : sc.strided_rows;
            const LineFactor& f = m.axis[a].factor;
            const size_t list = static_cast<size_t>(j) * kBatchClasses + batch_band_class(f.p, f.cyclic);
            values[list] += m.total * C;
            for (int ch = 0; ch < C; ++ch)
                for (int64_t l0 = 0; l0 < nlines; l0 += rows_max) {
                    SolveItem it{};
                    it.table = static_cast<int32_t>(i);
                    it.axis = static_cast<int16_t>(a);
                    it.contig = contig ? 1 : 0;
                    it.rows = static_cast<int32_t>(std::min<int64_t>(rows_max, nlines - l0));
                    it.chan = ch;
                    it.line0 = l0;
                    passes[list].push_back(it);
                }
        }
        for (int64_t s = 0; s < m.total * C; s += kChunkElems) {
            ChunkItem c{};
            c.table = static_cast<int32_t>(i);
            c.start = s;
            c.len = static_cast<int32_t>(std::min<int64_t>(kChunkElems, m.total * C - s));
            chunks.push_back(c);
        }
    }
    // longest lines first: the slowest warps start first
    auto longest_first = [&](const SolveItem& x, const SolveItem& y) {
        return b.models[x.table].axis[x.axis].n > b.models[y.table].axis[y.axis].n;
    };
    for (auto& p : passes) std::stable_sort(p.begin(), p.end(), longest_first);
}

// Builds and uploads the work lists of schedule sc (replacing the batch's).
intp_status apply_schedule(intp_batch* b, const intp_batch_schedule& sc) {
    if (sc.contig_rows < 1 || sc.contig_rows > 32 || sc.strided_rows < 1 || sc.strided_rows > 32)
        return bfail(INTP_ERR_INVALID_ARGUMENT, "schedule: contig_rows and strided_rows in [1, 32]");
    std::vector<std::vector<SolveItem>> passes;
    std::vector<int64_t> values;
    std::vector<ChunkItem> chunks;
    build_work(*b, sc, passes, values, chunks);
    Arena ar;
    std::vector<size_t> o_items(passes.size());
    for (size_t j = 0; j < passes.size(); ++j) o_items[j] = ar.put(passes[j]);
    if (b->work) cudaFree(b->work);
    b->work = nullptr;
    BATCH_CUDA(cudaMalloc(&b->work, std::max<size_t>(ar.host.size(), 16)), "cudaMalloc(batch work lists)");
    BATCH_CUDA(cudaMemcpy(b->work, ar.host.data(), ar.host.size(), cudaMemcpyHostToDevice), "cudaMemcpy(work lists)");
    const unsigned char* base = static_cast<const unsigned char*>(b->work);
    b->npasses = 0;
    for (int j = 0; j < kBatchMaxDim; ++j) {
        intp_batch::Pass& p = b->pass[j];
        p.nclasses = 0;
        for (int c = 0; c < kBatchClasses; ++c) {
            const size_t list = static_cast<size_t>(j) * kBatchClasses + c;
            p.items[c] = reinterpret_cast<const SolveItem*>(base + o_items[list]);
            p.nitems[c] = static_cast<int64_t>(passes[list].size());
            if (p.nitems[c] > 0) p.order[p.nclasses++] = c;
        }
        // the classes with the most values first
        std::stable_sort(p.order, p.order + p.nclasses, [&](int x, int y) {
            return values[static_cast<size_t>(j) * kBatchClasses + x] > values[static_cast<size_t>(j) * kBatchClasses + y];
        });
        if (p.nclasses > 0) b->npasses = j + 1;
    }
    b->sched = sc;
    b->sched.build_ms = 0.0;
    ++b->work_version;
    return INTP_OK;
}

int batch_sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    }
    return n;
}

// Streams and events for `need` concurrent side launches.
cudaError_t ensure_side_streams(intp_batch* b, int need) {
    if (need > 0 && !b->fork) {
        cudaError_t e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
        if (e != cudaSuccess) return e;
    }
    while (b->nside < need) {
        cudaStream_t st = nullptr;
        cudaEvent_t ev = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e != cudaSuccess) return e;
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            cudaStreamDestroy(st);
            return e;
        }
        b->side[b->nside] = st;
        b->join[b->nside] = ev;
        ++b->nside;
    }
    return cudaSuccess;
}

// One solve of every table: the axis passes in order; within a pass a launch
// per band class present, the classes concurrently (they touch disjoint
// tables) and joined before the next pass. `launch` numbers the persistent
// launches of the build (their work counters were cleared when the build
// started).
template <class R>
cudaError_t run_passes(intp_batch* b, R* data, int sel, int& launch, cudaStream_t s) {
    for (int j = 0; j < b->npasses; ++j) {
        const intp_batch::Pass& p = b->pass[j];
        if (p.nclasses == 0) continue;
        cudaError_t e = ensure_side_streams(b, p.nclasses - 1);
        if (e != cudaSuccess) return e;
        if (p.nclasses > 1) {
            e = cudaEventRecord(b->fork, s);
            if (e != cudaSuccess) return e;
        }
        for (int k = 0; k < p.nclasses; ++k) {
            const int c = p.order[k];
            cudaStream_t sk = k == 0 ? s : b->side[k - 1];
            if (k > 0) {
                e = cudaStreamWaitEvent(sk, b->fork, 0);
                if (e != cudaSuccess) return e;
            }
            BatchSolveLaunch a{};
            a.items = p.items[c];
            a.nitems = p.nitems[c];
            a.persistent = b->sched.persistent && launch < kMaxLaunches;
            a.counter = a.persistent ? b->counters + launch++ : nullptr;
            a.tables = b->d_tables;
            a.fac = b->d_fac;
            a.off = b->d_off;
            a.refine = b->d_refine;
            a.sel = sel;
            a.sm_count = batch_sm_count();
            e = launch_batch_solve(data, c, a, sk);
            if (e != cudaSuccess) return e;
            if (k > 0) {
                e = cudaEventRecord(b->join[k - 1], sk);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(s, b->join[k - 1], 0);
                if (e != cudaSuccess) return e;
            }
        }
    }
    return cudaSuccess;
}

intp_status batch_interpolate(intp_batch* b, const double* values, cudaStream_t s) {
    const int64_t N = b->off[b->ntables];
    int launch = 0;
    if (b->sched.persistent)
        BATCH_CUDA(cudaMemsetAsync(b->counters, 0, sizeof(unsigned int) * kMaxLaunches, s), "cudaMemsetAsync(counters)");
    const unsigned nch = static_cast<unsigned>(b->nchunks);
    if (!b->mixed()) {
        double* c = static_cast<double*>(b->ctrl);
        batch_elementwise_kernel<double><<<nch, 256, 0, s>>>(0, values, c, nullptr, nullptr, b->d_chunks, b->d_tables,
                                                             b->d_off, b->d_refine);
        note_launch();
        BATCH_CUDA(cudaGetLastError(), "batch shift copy");
        BATCH_CUDA(run_passes<double>(b, c, kBatchSelAll, launch, s), "batch line solve (fp64)");
        b->has_ctrl = true;
        return INTP_OK;
    }
    // mixed: the tables with refine = 0 solve in FP32 in place; the others
    // (all by default) in double-word arithmetic on a working array, split
    // into (ctrl, ctrl_lo) at the end -- the single-table solve's operations
    float* c = static_cast<float*>(b->ctrl);
    DW* w = nullptr;
    if (b->max_refine > 0) {
        const size_t need = static_cast<size_t>(N) * sizeof(DW) + 1024;
        if (b->scratch_bytes < need) {
            if (b->scratch) cudaFree(b->scratch);
            b->scratch = nullptr;
            b->scratch_bytes = 0;
            BATCH_CUDA(cudaMalloc(&b->scratch, need), "cudaMalloc(batch double-word scratch)");
            b->scratch_bytes = need;
        }
        w = static_cast<DW*>(b->scratch);
    }
    batch_elementwise_kernel<float><<<nch, 256, 0, s>>>(0, values, c, w, nullptr, b->d_chunks, b->d_tables, b->d_off,
                                                        b->d_refine);
    note_launch();
    BATCH_CUDA(cudaGetLastError(), "batch shift copy");
    if (b->min_refine == 0)
        BATCH_CUDA(run_passes<float>(b, c, kBatchSelPlain, launch, s), "batch line solve (fp32)");
    if (w) {
        BATCH_CUDA(run_passes<DW>(b, w, kBatchSelDW, launch, s), "batch line solve (double-word)");
        batch_elementwise_kernel<float><<<nch, 256, 0, s>>>(1, nullptr, c, w, b->ctrl_lo, b->d_chunks, b->d_tables,
                                                            b->d_off, b->d_refine);
        note_launch();
        BATCH_CUDA(cudaGetLastError(), "batch double-word split");
    }
    b->has_ctrl = true;
    return INTP_OK;
}

// The evaluation's work list: runs of at most kEvalRun points of one table,
// grouped by (dimension, order) class, with each class's plan.
struct EvalWork {
    std::vector<EvalItem> items;  // classes one after another
    struct Class {
        int D, O;
        size_t pos, count;
        DerivPlan plan;
    };
    std::vector<Class> classes;
    int64_t npts = 0;
    bool out_f32 = true;
};

intp_status make_eval_work(const intp_batch* b, const int64_t* point_offsets, const int32_t* derivs, int32_t nderiv,
                           int32_t out_dtype, EvalWork& w) {
    if (out_dtype != INTP_F64 && out_dtype != INTP_F32) return bfail(INTP_ERR_INVALID_ARGUMENT, "unknown output dtype");
    if (point_offsets[0] != 0) return bfail(INTP_ERR_INVALID_ARGUMENT, "point_offsets[0] must be 0");
    if (derivs && (nderiv < 1 || nderiv > INTP_GPU_MAX_DERIV))
        return bfail(INTP_ERR_INVALID_ARGUMENT, "nderiv must be in [1, 16]");
    w.out_f32 = out_dtype == INTP_F32;
    // runs of queries per (dim, order) class; table i's outputs follow those
    // of the tables before it, (points x K x channels) each
    std::vector<EvalItem> items[kBatchMaxDim + 1][INTP_GPU_MAX_ORDER + 1];
    const int64_t K = derivs ? nderiv : 1;
    int64_t coff = 0, ooff = 0;
    for (int64_t i = 0; i < b->ntables; ++i) {
        const int64_t p0 = point_offsets[i], p1 = point_offsets[i + 1];
        if (p1 < p0) return bfail(INTP_ERR_INVALID_ARGUMENT, "point_offsets must not decrease");
        const TableModel& m = b->models[i];
        for (int64_t p = p0; p < p1; p += kEvalRun) {
            EvalItem it{};
            it.table = static_cast<int32_t>(i);
            it.count = static_cast<int32_t>(std::min<int64_t>(kEvalRun, p1 - p));
            it.coord_off = coff + (p - p0) * m.dim;
            it.out_elem = ooff + (p - p0) * K * b->channels[i];
            items[m.dim][m.order].push_back(it);
        }
        coff += (p1 - p0) * m.dim;
        ooff += (p1 - p0) * K * b->channels[i];
    }
    w.npts = point_offsets[b->ntables];
    for (int D = 1; D <= kBatchMaxDim; ++D)
        for (int O = 0; O <= INTP_GPU_MAX_ORDER; ++O) {
            const std::vector<EvalItem>& v = items[D][O];
            if (v.empty()) continue;
            EvalWork::Class c{D, O, w.items.size(), v.size(), DerivPlan{}};
            std::string err;
            if (!build_deriv_plan(D, O, derivs, nderiv, INTP_GPU_MAX_DIM, c.plan, err))
                return bfail(INTP_ERR_INVALID_ARGUMENT, err);
            w.items.insert(w.items.end(), v.begin(), v.end());
            w.classes.push_back(c);
        }
    return INTP_OK;
}

// One launch per class of the work list (d_items: its device copy).
intp_status launch_eval_work(const intp_batch* b, const EvalWork& w, const EvalItem* d_items, const double* coords,
                             void* out, cudaStream_t s) {
    for (const EvalWork::Class& c : w.classes) {
        const cudaError_t e = launch_batch_eval(c.D, c.O, b->mixed(), b->d_tables, d_items + c.pos,
                                                static_cast<int64_t>(c.count), coords, c.plan, out, w.out_f32, s);
        if (e != cudaSuccess) return bcuda(e, "batched evaluation");
    }
    return INTP_OK;
}

}  // namespace

extern "C" {

intp_status intp_batch_create(const intp_table_desc* descs, int64_t ntables, intp_batch** out) {
    if (!descs || !out) return bfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (ntables < 1 || ntables > (int64_t{1} << 30)) return bfail(INTP_ERR_INVALID_ARGUMENT, "ntables must be >= 1");
    const int prec = descs[0].precision;
    if (prec != INTP_PRECISION_FP64 && prec != INTP_PRECISION_MIXED)
        return bfail(INTP_ERR_INVALID_ARGUMENT, "unknown precision");
    intp_batch* b = new (std::nothrow) intp_batch();
    if (!b) return bfail(INTP_ERR_OUT_OF_MEMORY, "out of host memory");
    b->precision = prec;
    b->ntables = ntables;
    b->off.assign(static_cast<size_t>(ntables) + 1, 0);
    b->refine.assign(static_cast<size_t>(ntables), 0);
    try {
        b->models.resize(static_cast<size_t>(ntables));
        b->channels.assign(static_cast<size_t>(ntables), 1);
        for (int64_t i = 0; i < ntables; ++i) {
            const intp_table_desc& d = descs[i];
            const std::string where = "table " + std::to_string(i) + ": ";
            if (d.precision != prec) {
                delete b;
                return bfail(INTP_ERR_INVALID_ARGUMENT, where + "every table of a batch has the same precision");
            }
            if (d.dim < 1 || d.dim > kBatchMaxDim) {
                delete b;
                return bfail(INTP_ERR_UNSUPPORTED, where + "batched tables have dimension 1..3");
            }
            if (d.channels < 0 || d.channels > INTP_GPU_MAX_CHANNELS) {
                delete b;
                return bfail(INTP_ERR_INVALID_ARGUMENT, where + "channels must be in [0, 64]");
            }
            if (d.order < 0 || d.order > INTP_GPU_MAX_ORDER) {
                delete b;
                return bfail(INTP_ERR_UNSUPPORTED, where + "order must be in [0, 7]");
            }
            if (d.refine_steps < -1 || d.refine_steps > 4) {
                delete b;
                return bfail(INTP_ERR_INVALID_ARGUMENT, where + "refine_steps must be in [-1, 4]");
            }
            TableSpec spec;
            spec.dim = d.dim;
            spec.order = d.order;
            for (int a = 0; a < d.dim; ++a) {
                spec.periodic[a] = d.periodic[a] != 0;
                spec.size[a] = d.size[a];
                spec.lo[a] = d.range_lo[a];
                spec.hi[a] = d.range_hi[a];
                spec.coords[a] = d.coords[a];
            }
            const std::string err = build_model(spec, b->models[i]);
            if (!err.empty()) {
                delete b;
                return bfail(INTP_ERR_INVALID_ARGUMENT, where + err);
            }
            for (int a = 0; a < d.dim; ++a) {
                const LineFactor& f = b->models[i].axis[a].factor;
                if (f.p != f.q || f.p > (f.cyclic ? kBatchMaxCyclicBand : kBatchMaxBand)) {
                    delete b;
                    return bfail(INTP_ERR_UNSUPPORTED, where + "band outside the batched solve's classes");
                }
            }
            b->channels[i] = d.channels > 1 ? d.channels : 1;
            if (b->models[i].total * b->channels[i] >= (int64_t{1} << 31)) {
                delete b;
                return bfail(INTP_ERR_UNSUPPORTED, where + "batched tables hold fewer than 2^31 values each");
            }
            b->off[i + 1] = b->off[i] + b->models[i].total * b->channels[i];
            if (b->mixed()) {
                b->refine[i] = d.refine_steps == 0 ? 0 : 1;
                b->max_refine = std::max(b->max_refine, b->refine[i]);
                b->min_refine = std::min(b->min_refine, b->refine[i]);
            }
        }
    } catch (const std::bad_alloc&) {
        delete b;
        return bfail(INTP_ERR_OUT_OF_MEMORY, "out of host memory");
    }
    cudaGetDevice(&b->device);

    // one arena: per-axis data of every table, then descriptors and work lists
    Arena ar;
    std::vector<PackedTable> packed(static_cast<size_t>(ntables));
    for (int64_t i = 0; i < ntables; ++i) pack_table(b->models[i], ar, packed[i]);
    std::vector<std::vector<SolveItem>> passes;
    std::vector<int64_t> pass_values;
    std::vector<ChunkItem> chunks;
    build_work(*b, b->sched, passes, pass_values, chunks);
    std::vector<int32_t> refine32(b->refine.begin(), b->refine.end());
    const size_t o_tables = ar.add(sizeof(TableDev) * static_cast<size_t>(ntables));
    const size_t o_fac = ar.add(sizeof(AxisFactorDev) * static_cast<size_t>(ntables) * kBatchMaxDim);
    const size_t o_off = ar.put(b->off);
    const size_t o_ref = ar.put(refine32);
    const size_t o_chunks = ar.put(chunks);
    cudaError_t e = cudaMalloc(&b->arena, ar.host.size());
    if (e != cudaSuccess) {
        delete b;
        return bcuda(e, "cudaMalloc(batch arena)");
    }
    const size_t N = static_cast<size_t>(b->off[ntables]);
    e = cudaMalloc(&b->ctrl, std::max<size_t>(N, 1) * b->elem());
    if (e == cudaSuccess && b->max_refine > 0)
        e = cudaMalloc(reinterpret_cast<void**>(&b->ctrl_lo), std::max<size_t>(N, 1) * sizeof(float));
    if (e != cudaSuccess) {
        delete b;
        return bcuda(e, "cudaMalloc(batch control points)");
    }
    const unsigned char* base = static_cast<const unsigned char*>(b->arena);
    b->h_tables.resize(static_cast<size_t>(ntables));
    std::vector<AxisFactorDev> fac(static_cast<size_t>(ntables) * kBatchMaxDim);
    for (int64_t i = 0; i < ntables; ++i) {
        double lo_user[kMaxDim] = {};
        for (int a = 0; a < descs[i].dim; ++a) lo_user[a] = descs[i].range_lo[a];
        TableDev& dv = b->h_tables[i];
        std::memset(&dv, 0, sizeof dv);
        bind_table(b->models[i], lo_user, packed[i], base, dv, &fac[i * kBatchMaxDim]);
        dv.channels = b->channels[i];
        dv.ctrl = static_cast<const unsigned char*>(b->ctrl) + static_cast<size_t>(b->off[i]) * b->elem();
        dv.ctrl_lo = b->refine[i] > 0 ? b->ctrl_lo + b->off[i] : nullptr;
    }
    std::memcpy(ar.host.data() + o_tables, b->h_tables.data(), sizeof(TableDev) * static_cast<size_t>(ntables));
    std::memcpy(ar.host.data() + o_fac, fac.data(), sizeof(AxisFactorDev) * fac.size());
    e = cudaMemcpy(b->arena, ar.host.data(), ar.host.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        delete b;
        return bcuda(e, "cudaMemcpy(batch arena)");
    }
    b->d_tables = reinterpret_cast<TableDev*>(static_cast<unsigned char*>(b->arena) + o_tables);
    b->d_fac = reinterpret_cast<const AxisFactorDev*>(base + o_fac);
    b->d_off = reinterpret_cast<const int64_t*>(base + o_off);
    b->d_refine = reinterpret_cast<const int32_t*>(base + o_ref);
    b->d_chunks = reinterpret_cast<const ChunkItem*>(base + o_chunks);
    b->nchunks = static_cast<int64_t>(chunks.size());
    e = cudaMalloc(reinterpret_cast<void**>(&b->counters), sizeof(unsigned int) * kMaxLaunches);
    if (e != cudaSuccess) {
        delete b;
        return bcuda(e, "cudaMalloc(batch work counters)");
    }
    const intp_status st = apply_schedule(b, b->sched);
    if (st != INTP_OK) {
        delete b;
        return st;
    }
    *out = b;
    return INTP_OK;
}

intp_status intp_batch_destroy(intp_batch* b) {
    delete b;
    return INTP_OK;
}

intp_status intp_batch_info(const intp_batch* b, int64_t* ntables, int64_t* total_values) {
    if (!b) return bfail(INTP_ERR_INVALID_ARGUMENT, "null batch");
    if (ntables) *ntables = b->ntables;
    if (total_values) *total_values = b->off[b->ntables];
    return INTP_OK;
}

intp_status intp_batch_build(intp_batch* b, const double* values, int32_t values_on_device, void* stream) {
    if (!b || !values) return bfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (values_on_device) return batch_interpolate(b, values, s);
    const size_t bytes = static_cast<size_t>(b->off[b->ntables]) * 8;
    void* stage = nullptr;
    BATCH_CUDA(cudaMallocAsync(&stage, bytes, s), "cudaMallocAsync(batch values)");
    cudaError_t e = cudaMemcpyAsync(stage, values, bytes, cudaMemcpyHostToDevice, s);
    intp_status st = e == cudaSuccess ? batch_interpolate(b, static_cast<double*>(stage), s)
                                      : bcuda(e, "cudaMemcpyAsync(batch values)");
    cudaFreeAsync(stage, s);
    return st;
}

intp_status intp_batch_set_schedule(intp_batch* b, const intp_batch_schedule* sc) {
    if (!b || !sc) return bfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    return apply_schedule(b, *sc);
}

intp_status intp_batch_get_schedule(const intp_batch* b, intp_batch_schedule* sc) {
    if (!b || !sc) return bfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    *sc = b->sched;
    return INTP_OK;
}

intp_status intp_batch_autotune(intp_batch* b, const double* values, int32_t values_on_device, void* stream,
                                intp_batch_schedule* chosen) {
    if (!b || !values) return bfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the values on the device once, so the timings are of the builds alone
    const double* v = values;
    void* stage = nullptr;
    if (!values_on_device) {
        const size_t bytes = static_cast<size_t>(b->off[b->ntables]) * 8;
        BATCH_CUDA(cudaMalloc(&stage, bytes), "cudaMalloc(autotune values)");
        cudaError_t e = cudaMemcpy(stage, values, bytes, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(stage);
            return bcuda(e, "cudaMemcpy(autotune values)");
        }
        v = static_cast<const double*>(stage);
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    intp_status st = INTP_OK;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        st = bfail(INTP_ERR_CUDA, "cudaEventCreate");
    intp_batch_schedule best{};
    double best_ms = 0.0;
    const int32_t crows[] = {16, 32};
    const int32_t rows[] = {16, 32};
    for (int pers = 0; pers < 2 && st == INTP_OK; ++pers)
        for (int32_t cr : crows)
            for (int32_t r : rows) {
                if (st != INTP_OK) break;
                intp_batch_schedule sc{pers, cr, r, 0, 0.0};
                st = apply_schedule(b, sc);
                if (st == INTP_OK) st = batch_interpolate(b, v, s);  // warm-up
                if (st != INTP_OK) break;
                cudaEventRecord(e0, s);
                for (int rep = 0; rep < 2 && st == INTP_OK; ++rep) st = batch_interpolate(b, v, s);
                cudaEventRecord(e1, s);
                if (cudaEventSynchronize(e1) != cudaSuccess) st = bfail(INTP_ERR_CUDA, "autotune timing");
                if (st != INTP_OK) break;
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                sc.build_ms = ms / 2.0;
                if (best_ms == 0.0 || sc.build_ms < best_ms) {
                    best = sc;
                    best_ms = sc.build_ms;
                }
            }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st == INTP_OK) st = apply_schedule(b, best);
    if (st == INTP_OK) {
        b->sched.build_ms = best_ms;
        // the batch holds the control points of the chosen schedule's build
        st = batch_interpolate(b, v, s);
        if (st == INTP_OK && cudaStreamSynchronize(s) != cudaSuccess) st = bfail(INTP_ERR_CUDA, "autotune build");
    }
    if (stage) cudaFree(stage);
    if (st == INTP_OK && chosen) *chosen = b->sched;
    return st;
}

intp_status intp_batch_get_control_points(const intp_batch* b, int64_t table, double* out) {
    if (!b || !out) return bfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    if (table < 0 || table >= b->ntables) return bfail(INTP_ERR_INVALID_ARGUMENT, "table index out of range");
    if (!b->has_ctrl) return bfail(INTP_ERR_STATE, "batch has no control points yet");
    const int64_t n = b->off[table + 1] - b->off[table];
    BATCH_CUDA(cudaDeviceSynchronize(), "synchronize");
    const unsigned char* src = static_cast<const unsigned char*>(b->ctrl) + static_cast<size_t>(b->off[table]) * b->elem();
    if (b->mixed()) {
        const bool lo = b->refine[table] > 0;
        std::vector<float> f(static_cast<size_t>(n)), r(lo ? static_cast<size_t>(n) : 0);
        BATCH_CUDA(cudaMemcpy(f.data(), src, static_cast<size_t>(n) * 4, cudaMemcpyDeviceToHost), "cudaMemcpy(ctrl)");
        if (lo)
            BATCH_CUDA(cudaMemcpy(r.data(), b->ctrl_lo + b->off[table], static_cast<size_t>(n) * 4,
                                  cudaMemcpyDeviceToHost),
                       "cudaMemcpy(ctrl)");
        for (int64_t i = 0; i < n; ++i) out[i] = static_cast<double>(f[i]) + (lo ? static_cast<double>(r[i]) : 0.0);
    } else {
        BATCH_CUDA(cudaMemcpy(out, src, static_cast<size_t>(n) * 8, cudaMemcpyDeviceToHost), "cudaMemcpy(ctrl)");
    }
    // vector-valued tables: from one mesh per channel to channel fastest,
    // as intp_table_get_control_points gives them
    const int64_t C = b->channels[table];
    if (C > 1) {
        const int64_t P = n / C;
        std::vector<double> planar(out, out + n);
        for (int64_t i = 0; i < P; ++i)
            for (int64_t c = 0; c < C; ++c) out[i * C + c] = planar[c * P + i];
    }
    return INTP_OK;
}

intp_status intp_batch_eval(const intp_batch* b, const double* coords, const int64_t* point_offsets,
                            const int32_t* derivs, int32_t nderiv, void* out, int32_t out_dtype, void* stream) {
    if (!b || !point_offsets) return bfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    if (!b->has_ctrl) return bfail(INTP_ERR_STATE, "batch has no control points yet");
    EvalWork w;
    intp_status st = make_eval_work(b, point_offsets, derivs, nderiv, out_dtype, w);
    if (st != INTP_OK || w.npts == 0) return st;
    if (!coords || !out) return bfail(INTP_ERR_INVALID_ARGUMENT, "null buffer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    EvalItem* d_items = nullptr;
    BATCH_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&d_items), w.items.size() * sizeof(EvalItem), s),
               "cudaMallocAsync(batch work list)");
    cudaError_t e = cudaMemcpyAsync(d_items, w.items.data(), w.items.size() * sizeof(EvalItem), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) st = bcuda(e, "cudaMemcpyAsync(batch work list)");
    if (st == INTP_OK) st = launch_eval_work(b, w, d_items, coords, out, s);
    cudaFreeAsync(d_items, s);
    return st;
}

// A captured build + evaluation: the evaluation's work list uploaded once,
// then one intp_batch_build and one intp_batch_eval recorded on a capturing
// stream (the build's side streams join the capture through its events).
struct intp_batch_graph {
    intp_batch* b = nullptr;
    uint64_t work_version = 0;  // the batch's work lists the capture reads
    void* items = nullptr;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~intp_batch_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (cap) cudaStreamDestroy(cap);
        if (items) cudaFree(items);
    }
};

intp_status intp_batch_graph_create(intp_batch* b, const double* values, const double* coords,
                                    const int64_t* point_offsets, const int32_t* derivs, int32_t nderiv, void* out,
                                    int32_t out_dtype, intp_batch_graph** out_graph) {
    if (!b || !values || !point_offsets || !out_graph) return bfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    *out_graph = nullptr;
    EvalWork w;
    intp_status st = make_eval_work(b, point_offsets, derivs, nderiv, out_dtype, w);
    if (st != INTP_OK) return st;
    if (w.npts > 0 && (!coords || !out)) return bfail(INTP_ERR_INVALID_ARGUMENT, "null buffer");
    intp_batch_graph* g = new (std::nothrow) intp_batch_graph();
    if (!g) return bfail(INTP_ERR_OUT_OF_MEMORY, "out of host memory");
    g->b = b;
    auto gfail = [&](intp_status code) {
        delete g;
        return code;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&g->cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) return gfail(bcuda(e, "cudaStreamCreate(capture)"));
    if (!w.items.empty()) {
        e = cudaMalloc(&g->items, w.items.size() * sizeof(EvalItem));
        if (e == cudaSuccess)
            e = cudaMemcpy(g->items, w.items.data(), w.items.size() * sizeof(EvalItem), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return gfail(bcuda(e, "batch graph work list"));
    }
    // one build outside the capture: it sets up the solve's working array and
    // the side streams, which a capture may not create
    st = batch_interpolate(b, values, g->cap);
    if (st != INTP_OK) return gfail(st);
    e = cudaStreamSynchronize(g->cap);
    if (e != cudaSuccess) return gfail(bcuda(e, "batch graph warm-up build"));
    e = cudaStreamBeginCapture(g->cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return gfail(bcuda(e, "cudaStreamBeginCapture"));
    st = batch_interpolate(b, values, g->cap);
    if (st == INTP_OK && w.npts > 0)
        st = launch_eval_work(b, w, static_cast<const EvalItem*>(g->items), coords, out, g->cap);
    e = cudaStreamEndCapture(g->cap, &g->graph);
    if (st != INTP_OK) return gfail(st);
    if (e != cudaSuccess) return gfail(bcuda(e, "cudaStreamEndCapture"));
    e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    if (e != cudaSuccess) return gfail(bcuda(e, "cudaGraphInstantiate"));
    g->work_version = b->work_version;
    *out_graph = g;
    return INTP_OK;
}

intp_status intp_batch_graph_launch(intp_batch_graph* g, void* stream) {
    if (!g) return bfail(INTP_ERR_INVALID_ARGUMENT, "null graph");
    // a new schedule replaced the work lists the capture reads
    if (g->work_version != g->b->work_version)
        return bfail(INTP_ERR_STATE, "the batch's schedule changed after the graph was captured");
    BATCH_CUDA(cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream)), "cudaGraphLaunch");
    g->b->has_ctrl = true;
    return INTP_OK;
}

intp_status intp_batch_graph_destroy(intp_batch_graph* g) {
    delete g;
    return INTP_OK;
}

}  // extern "C"
