// Serving loop: one worker thread keeps built tables resident in HBM and runs
// table-build and evaluate requests of mixed sizes with continuous batching.
//
// Requests are submitted from any host thread and return at once with a
// request id. The worker admits queued requests whenever a slot (a CUDA
// stream with its completion event) and device memory are free:
//   - a build creates the table with stream-ordered allocations on the slot's
//     stream, copies the values in and solves the control points;
//   - evaluations queued against the same table (same derivative request and
//     output type) are merged into one work unit: their coordinates are copied
//     into one device buffer, evaluated by one intp_eval, and each request's
//     results are copied back to its own host buffer;
//   - an evaluation larger than a work unit (kPiecePoints) is split into
//     pieces, each its own unit; the request completes with its last piece.
// Work units on different slots overlap on the device; requests that arrive
// while others run are admitted as soon as a slot and memory free up, without
// waiting for the running ones to drain. A quarter of the slots (at least one
// when there are two or more) take small requests only (evaluations of up to
// kSmallPoints points, builds of up to kSmallValues values) and run on
// high-priority streams, so that small requests neither queue behind large
// ones for a slot nor wait for their kernels on the device.
//
// Memory: resident tables plus the transient bytes of the work in flight stay
// within the configured budget. At creation the server reserves
// min(budget, kPoolReserve) in the device's stream-ordered pool (freed
// memory stays in the pool), so admissions carve from it instead of waiting
// for new memory to be mapped while other requests queue. A unit that does not fit evicts the least
// recently used resident tables that no queued or running request refers to;
// when that is not enough it waits for running units to finish, and fails
// with INTP_ERR_BUDGET when it could never fit.
//
// Latency of a request is measured from its submission to the completion of
// its work unit on the device; the stats report p50/p99 and points per second.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <iterator>
#include <list>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "intp_gpu.h"
#include "table_internal.hpp"
#include "table_pack.hpp"

using namespace intp_gb300;

namespace {

using Clock = std::chrono::steady_clock;

constexpr int kMaxSlots = 64;
constexpr uint64_t kDefaultBudget = uint64_t{150} << 30;
constexpr int64_t kDefaultMaxBatchPoints = int64_t{1} << 24;
// transient bytes of the binned evaluation (batches of at least
// kBinnedPoints queries): per query its 16-byte sort record, plus an
// allowance for the per-bucket bookkeeping
constexpr size_t kEvalScratchPerPoint = 16;
constexpr size_t kEvalScratchFixed = size_t{16} << 20;
constexpr int64_t kBinnedPoints = int64_t{1} << 18;
// work-unit bounds: the largest evaluation unit (larger requests are split),
// and what counts as small for the reserved slots
constexpr int64_t kPiecePoints = int64_t{1} << 21;
constexpr int64_t kSmallPoints = int64_t{1} << 16;
constexpr int64_t kSmallValues = int64_t{1} << 18;
// device memory reserved in the stream-ordered pool at creation (at most the
// budget): tables and work units are carved from it, so an admission does not
// wait for the driver to map new memory while requests queue behind it
constexpr uint64_t kPoolReserve = uint64_t{64} << 30;

size_t eval_reserve(int64_t npts, size_t per_point) {
    return static_cast<size_t>(npts) * per_point + (npts >= kBinnedPoints ? kEvalScratchFixed : 0);
}

enum TableState : int32_t { kQueued = 0, kResident = 1, kGone = 2, kFailed = 3 };

struct Request {
    int64_t id = 0;
    bool build = false;
    int64_t table = 0;
    // build
    intp_table_desc desc{};
    std::vector<double> axis_coords[INTP_GPU_MAX_DIM];  // non-uniform axes, copied at submission
    const double* values = nullptr;
    // evaluation
    const double* coords = nullptr;
    int64_t npts = 0;
    std::vector<int32_t> derivs;
    int32_t nderiv = 0;
    void* out = nullptr;
    int32_t out_dtype = INTP_F32;
    int64_t admitted = 0;  // points placed into work units so far
    int parts_open = 0;    // work units in flight holding a piece of it
    // result
    Clock::time_point t_submit;
    Clock::time_point t_admit;  // its first work unit was issued
    double device_ms = 0.0;     // tracing: device time of its work units (sum)
    bool admitted_once = false;
    intp_status status = INTP_OK;
    std::string error;
    bool done = false;
};

struct Table {
    intp_table* t = nullptr;
    int32_t state = kQueued;
    int dim = 0;
    int channels = 1;       // values per mesh point (vector-valued tables)
    int refs = 0;           // queued or running requests that use the table
    bool release = false;   // drop once refs reaches 0
    size_t bytes = 0;       // device bytes while resident
    uint64_t last_use = 0;  // LRU clock
};

// Points [off, off + n) of an evaluation request (a build: its whole request).
struct Part {
    Request* r = nullptr;
    int64_t off = 0, n = 0;
};

struct Unit {
    bool build = false;
    std::vector<Part> parts;
    int64_t table = 0;
    size_t reserve = 0;  // transient device bytes counted while in flight
    int64_t npts = 0;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    cudaEvent_t start = nullptr;  // tracing: recorded when a unit is issued (timing events)
    bool busy = false;
    bool small_only = false;  // reserved for small requests (high-priority stream)
    Unit unit;
};

int64_t build_values(const intp_table_desc& d) {
    int64_t n = d.channels > 1 ? d.channels : 1;
    for (int k = 0; k < d.dim; ++k) n *= d.size[k];
    return n;
}

double ms_since(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

bool is_device_pointer(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

double percentile(std::vector<double> v, double q) {
    if (v.empty()) return 0.0;
    const size_t k = static_cast<size_t>(q * static_cast<double>(v.size() - 1) + 0.5);
    std::nth_element(v.begin(), v.begin() + static_cast<std::ptrdiff_t>(k), v.end());
    return v[k];
}

}  // namespace

struct intp_server {
    int device = 0;
    uint64_t budget = kDefaultBudget;
    int64_t max_batch_points = kDefaultMaxBatchPoints;
    std::vector<Slot> slots;

    std::mutex mu;
    std::condition_variable cv_work;  // worker: new requests or stop
    std::condition_variable cv_done;  // waiters: a request completed
    bool stop = false;
    std::thread worker;

    int64_t next_request = 1;
    int64_t next_table = 1;
    std::list<Request*> pending;                        // submitted, not admitted
    std::unordered_map<int64_t, Request*> requests;     // every request not yet waited on
    std::unordered_map<int64_t, Table> tables;
    uint64_t lru_clock = 0;
    uint64_t resident_bytes = 0;
    uint64_t inflight_bytes = 0;

    // statistics since the last reset
    std::vector<double> lat_build, lat_eval;
    // request trace (INTP_GB300_SERVER_TRACE=<file>): one line per completed
    // request, written when the server is destroyed; its device_ms column
    // sums the device time of the request's work units
    std::string trace_path;
    std::vector<std::string> trace;
    // tracing: worker-loop iterations that began more than 5 ms after the
    // previous one (start ms, gap ms), written to <trace file>.gaps
    std::vector<std::pair<double, double>> loop_gaps;
    double points = 0;
    int64_t failed = 0, evictions = 0, merged_units = 0;
    Clock::time_point t_reset = Clock::now(), t_last = Clock::now();

    ~intp_server();
    void run();
    void finish_slot(Slot& s, cudaError_t e);
    bool admit(Slot& s, std::unique_lock<std::mutex>& lock);
    bool make_room(size_t need);
    void fail_request(Request* r, intp_status st, const std::string& msg);
    void complete(Request* r, intp_status st, const std::string& msg, Clock::time_point now);
    void drop_table(int64_t id, Table& tb);
};

namespace {

bool same_request_shape(const Request* a, const Request* b) {
    return a->table == b->table && a->out_dtype == b->out_dtype && a->nderiv == b->nderiv && a->derivs == b->derivs;
}

}  // namespace

void intp_server::complete(Request* r, intp_status st, const std::string& msg, Clock::time_point now) {
    if (!trace_path.empty()) {
        char line[256];
        const Clock::time_point ta = r->admitted_once ? r->t_admit : now;
        std::snprintf(line, sizeof line, "%lld,%d,%lld,%.3f,%.3f,%.3f,%.3f,%d\n", static_cast<long long>(r->id),
                      r->build ? 1 : 0, static_cast<long long>(r->build ? build_values(r->desc) : r->npts),
                      ms_since(t_reset, r->t_submit), ms_since(r->t_submit, ta), ms_since(ta, now), r->device_ms,
                      static_cast<int>(st));
        trace.emplace_back(line);
    }
    r->status = st;
    r->error = msg;
    r->done = true;
    cv_done.notify_all();  // waiters re-check under the lock the worker holds
    if (st == INTP_OK) {
        (r->build ? lat_build : lat_eval).push_back(ms_since(r->t_submit, now));
        if (!r->build) points += static_cast<double>(r->npts);
        t_last = now;
    } else {
        ++failed;
    }
    if (!r->build) {
        auto it = tables.find(r->table);
        if (it != tables.end()) {
            it->second.refs--;
            it->second.last_use = ++lru_clock;
            if (it->second.release && it->second.refs == 0) drop_table(it->first, it->second);
        }
    }
}

void intp_server::fail_request(Request* r, intp_status st, const std::string& msg) {
    complete(r, st, msg, Clock::now());
}

void intp_server::drop_table(int64_t id, Table& tb) {
    (void)id;
    if (tb.t) {
        intp_table_destroy(tb.t);  // stream-ordered frees on the table's build stream
        tb.t = nullptr;
    }
    if (tb.state == kResident) resident_bytes -= tb.bytes;
    tb.bytes = 0;
    tb.state = kGone;
}

// Evicts least recently used idle tables until `need` more bytes fit.
bool intp_server::make_room(size_t need) {
    while (resident_bytes + inflight_bytes + need > budget) {
        int64_t victim = -1;
        uint64_t oldest = ~uint64_t{0};
        for (auto& kv : tables) {
            const Table& tb = kv.second;
            if (tb.state == kResident && tb.refs == 0 && tb.last_use < oldest) {
                oldest = tb.last_use;
                victim = kv.first;
            }
        }
        if (victim < 0) return false;
        drop_table(victim, tables[victim]);
        ++evictions;
    }
    return true;
}

void intp_server::finish_slot(Slot& s, cudaError_t e) {
    const Clock::time_point now = Clock::now();
    Unit& u = s.unit;
    inflight_bytes -= u.reserve;
    if (s.start && e == cudaSuccess) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, s.start, s.done) == cudaSuccess)
            for (const Part& pt : u.parts) pt.r->device_ms += ms;
    }
    if (u.build) {
        Request* r = u.parts[0].r;
        Table& tb = tables[u.table];
        if (e == cudaSuccess && tb.t) {
            table_release_scratch(tb.t);
            tb.bytes = table_device_bytes(tb.t);
            tb.state = kResident;
            tb.last_use = ++lru_clock;
            resident_bytes += tb.bytes;
            complete(r, INTP_OK, "", now);
            if (tb.release && tb.refs == 0) drop_table(u.table, tb);
        } else {
            if (tb.t) intp_table_destroy(tb.t);
            tb.t = nullptr;
            tb.state = kFailed;
            complete(r, INTP_ERR_CUDA, std::string("table build: ") + cudaGetErrorString(e), now);
        }
    } else {
        for (const Part& pt : u.parts) {
            Request* r = pt.r;
            if (e != cudaSuccess && r->status == INTP_OK) {
                r->status = INTP_ERR_CUDA;
                r->error = std::string("evaluation: ") + cudaGetErrorString(e);
            }
            r->parts_open--;
            if (r->admitted == r->npts && r->parts_open == 0) complete(r, r->status, r->error, now);
        }
        if (u.parts.size() > 1) ++merged_units;
    }
    s.busy = false;
    s.unit = Unit{};
    cv_done.notify_all();
}

// Admits the first admissible pending request (with the evaluations that
// merge into it) onto slot s. Returns false when nothing could be admitted.
bool intp_server::admit(Slot& s, std::unique_lock<std::mutex>& lock) {
    (void)lock;
    for (auto it = pending.begin(); it != pending.end(); ++it) {
        Request* r = *it;
        // a reserved slot takes small requests only
        if (s.small_only && (r->build ? build_values(r->desc) > kSmallValues : r->npts - r->admitted > kSmallPoints))
            continue;
        if (r->build) {
            const size_t need = table_build_scratch_bytes(&r->desc) +
                                [&] {
                                    int64_t n = std::max(r->desc.channels, 1);
                                    for (int d = 0; d < r->desc.dim; ++d) n *= r->desc.size[d];
                                    return static_cast<size_t>(n) * 8 + (size_t{1} << 20);
                                }();
            if (need > budget) {
                pending.erase(it);
                tables[r->table].state = kFailed;
                fail_request(r, INTP_ERR_BUDGET, "table build exceeds the memory budget");
                return true;
            }
            if (!make_room(need)) continue;
            pending.erase(it);
            Unit u;
            u.build = true;
            u.parts.push_back(Part{r, 0, 0});
            r->t_admit = Clock::now();
            r->admitted_once = true;
            u.table = r->table;
            u.reserve = need;
            intp_table* t = nullptr;
            if (s.start) cudaEventRecord(s.start, s.stream);
            intp_status st = create_table(&r->desc, true, s.stream, &t);
            if (st == INTP_OK) {
                tables[r->table].t = t;
                st = intp_table_interpolate(t, r->values, is_device_pointer(r->values) ? 1 : 0, s.stream);
            }
            if (st != INTP_OK) {
                const std::string msg = intp_last_error();
                if (t) intp_table_destroy(t);
                tables[r->table].t = nullptr;
                tables[r->table].state = kFailed;
                fail_request(r, st, msg);
                return true;
            }
            inflight_bytes += need;
            cudaEventRecord(s.done, s.stream);
            s.unit = std::move(u);
            s.busy = true;
            return true;
        }
        // evaluation
        auto tt = tables.find(r->table);
        if (tt == tables.end() || tt->second.state == kGone || tt->second.state == kFailed) {
            pending.erase(it);
            fail_request(r, INTP_ERR_STATE, "table is not resident (evicted, released or failed)");
            return true;
        }
        if (tt->second.state != kResident) continue;  // its build has not finished
        Table& tb = tt->second;
        // the next piece of this request, then (while the unit has room) the
        // queued evaluations of the same shape that fit whole, in submission
        // order
        Unit u;
        u.table = r->table;
        // output values per point: one per derivative and channel
        const int K = (r->derivs.empty() ? 1 : r->nderiv) * tb.channels;
        const size_t ob = r->out_dtype == INTP_F32 ? 4 : 8;
        const size_t per_pt = static_cast<size_t>(tb.dim) * 8 + static_cast<size_t>(K) * ob + kEvalScratchPerPoint;
        const int64_t cap = std::min(max_batch_points, s.small_only ? kSmallPoints : kPiecePoints);
        u.parts.push_back(Part{r, r->admitted, std::min(r->npts - r->admitted, cap)});
        u.npts = u.parts[0].n;
        if (r->admitted + u.npts == r->npts) {
            for (auto jt = std::next(it); jt != pending.end() && u.npts < cap; ++jt) {
                Request* q = *jt;
                if (q->build || !same_request_shape(r, q) || q->admitted != 0 || u.npts + q->npts > cap) continue;
                u.parts.push_back(Part{q, 0, q->npts});
                u.npts += q->npts;
            }
        }
        u.reserve = eval_reserve(u.npts, per_pt);
        if (u.reserve > budget) {
            // a single piece too large for the budget on its own
            if (r->parts_open > 0) continue;  // wait for its other pieces, then fail
            pending.erase(it);
            r->admitted = r->npts;
            fail_request(r, INTP_ERR_BUDGET, "evaluation exceeds the memory budget");
            return true;
        }
        if (!make_room(u.reserve)) {
            // take the first piece alone if the merged unit does not fit
            if (u.parts.size() == 1) continue;
            u.parts.resize(1);
            u.npts = u.parts[0].n;
            u.reserve = eval_reserve(u.npts, per_pt);
            if (!make_room(u.reserve)) continue;
        }
        const Clock::time_point t_now = Clock::now();
        for (const Part& pt : u.parts) {
            if (!pt.r->admitted_once) {
                pt.r->t_admit = t_now;
                pt.r->admitted_once = true;
            }
            pt.r->admitted += pt.n;
            pt.r->parts_open++;
            if (pt.r->admitted == pt.r->npts) pending.remove(pt.r);
        }
        const int D = tb.dim;
        cudaStream_t st = s.stream;
        if (s.start) cudaEventRecord(s.start, st);
        double* dc = nullptr;
        void* dout = nullptr;
        cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&dc), static_cast<size_t>(u.npts) * D * 8 + 16, st);
        if (e == cudaSuccess) e = cudaMallocAsync(&dout, static_cast<size_t>(u.npts) * K * ob + 16, st);
        int64_t off = 0;
        for (const Part& pt : u.parts) {
            if (e != cudaSuccess) break;
            if (pt.n > 0)
                e = cudaMemcpyAsync(dc + off * D, pt.r->coords + pt.off * D, static_cast<size_t>(pt.n) * D * 8,
                                    cudaMemcpyDefault, st);
            off += pt.n;
        }
        intp_status ist = INTP_OK;
        std::string msg;
        if (e == cudaSuccess) {
            ist = intp_eval(tb.t, dc, u.npts, r->derivs.empty() ? nullptr : r->derivs.data(), r->nderiv, dout,
                            r->out_dtype, st);
            if (ist != INTP_OK) msg = intp_last_error();
        }
        off = 0;
        for (const Part& pt : u.parts) {
            if (e != cudaSuccess || ist != INTP_OK) break;
            if (pt.n > 0)
                e = cudaMemcpyAsync(static_cast<unsigned char*>(pt.r->out) + static_cast<size_t>(pt.off) * K * ob,
                                    static_cast<unsigned char*>(dout) + static_cast<size_t>(off) * K * ob,
                                    static_cast<size_t>(pt.n) * K * ob, cudaMemcpyDefault, st);
            off += pt.n;
        }
        if (dc) cudaFreeAsync(dc, st);
        if (dout) cudaFreeAsync(dout, st);
        if (e != cudaSuccess || ist != INTP_OK) {
            if (ist == INTP_OK) {
                ist = e == cudaErrorMemoryAllocation ? INTP_ERR_OUT_OF_MEMORY : INTP_ERR_CUDA;
                msg = std::string("evaluation: ") + cudaGetErrorString(e);
            }
            // copies already queued for earlier requests of the unit may still
            // be writing their outputs: the requests are reported done only
            // once the slot's stream has drained (and, for a split request,
            // once its other pieces have finished); their points not yet
            // admitted are dropped
            cudaStreamSynchronize(st);
            for (const Part& pt : u.parts) {
                Request* q = pt.r;
                if (q->status == INTP_OK) {
                    q->status = ist;
                    q->error = msg;
                }
                if (q->admitted < q->npts) {
                    q->admitted = q->npts;
                    pending.remove(q);
                }
                if (--q->parts_open == 0) complete(q, q->status, q->error, Clock::now());
            }
            return true;
        }
        tb.last_use = ++lru_clock;
        inflight_bytes += u.reserve;
        cudaEventRecord(s.done, st);
        s.unit = std::move(u);
        s.busy = true;
        return true;
    }
    return false;
}

void intp_server::run() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lock(mu);
    Clock::time_point t_prev = Clock::now();
    for (;;) {
        if (!trace_path.empty()) {
            const Clock::time_point t_it = Clock::now();
            const double gap = ms_since(t_prev, t_it);
            if (gap > 5.0) loop_gaps.emplace_back(ms_since(t_reset, t_it), gap);
            t_prev = t_it;
        }
        bool any_busy = false;
        for (Slot& s : slots) {
            if (!s.busy) continue;
            const cudaError_t q = cudaEventQuery(s.done);
            if (q != cudaErrorNotReady) finish_slot(s, q);
            any_busy = any_busy || s.busy;
        }
        bool admitted = false;
        for (Slot& s : slots) {
            if (s.busy || pending.empty()) continue;
            if (admit(s, lock)) admitted = true;
            any_busy = any_busy || s.busy;
        }
        if (stop && pending.empty() && !any_busy) break;
        if (stop && !any_busy && !admitted) {
            // shutting down with requests that can no longer be admitted
            // (waiting on memory or on a table that will not come)
            while (!pending.empty()) {
                Request* r = pending.front();
                pending.pop_front();
                if (r->build) tables[r->table].state = kFailed;
                r->admitted = r->npts;
                if (r->parts_open == 0)  // always so: no unit is in flight
                    fail_request(r, INTP_ERR_STATE, "server shut down before the request could run");
            }
            continue;
        }
        if (admitted) continue;
        if (any_busy) {
            // poll the running units' events
            lock.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
            lock.lock();
        } else {
            cv_work.wait_for(lock, std::chrono::milliseconds(2));
        }
    }
}

intp_server::~intp_server() {
    {
        std::lock_guard<std::mutex> g(mu);
        stop = true;
    }
    cv_work.notify_all();
    if (worker.joinable()) worker.join();
    cudaSetDevice(device);
    for (auto& kv : tables)
        if (kv.second.t) intp_table_destroy(kv.second.t);
    for (Slot& s : slots) {
        if (s.stream) cudaStreamSynchronize(s.stream);
        if (s.done) cudaEventDestroy(s.done);
        if (s.start) cudaEventDestroy(s.start);
        if (s.stream) cudaStreamDestroy(s.stream);
    }
    for (auto& kv : requests) delete kv.second;  // includes any never waited on
    if (!trace_path.empty()) {
        if (FILE* f = std::fopen(trace_path.c_str(), "w")) {
            std::fputs("id,build,size,submit_ms,queue_ms,service_ms,device_ms,status\n", f);
            for (const std::string& l : trace) std::fputs(l.c_str(), f);
            std::fclose(f);
        }
        if (FILE* f = std::fopen((trace_path + ".gaps").c_str(), "w")) {
            std::fputs("at_ms,gap_ms\n", f);
            for (const auto& g : loop_gaps) std::fprintf(f, "%.3f,%.3f\n", g.first, g.second);
            std::fclose(f);
        }
    }
}

namespace {

intp_status sfail(intp_status s, const std::string& msg) {
    set_last_error(msg);
    return s;
}

}  // namespace

extern "C" {

intp_status intp_server_create(const intp_server_config* cfg, intp_server** out) {
    if (!out) return sfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    intp_server_config c{};
    if (cfg) c = *cfg;
    const int nslots = c.slots > 0 ? c.slots : 4;
    if (nslots > kMaxSlots) return sfail(INTP_ERR_INVALID_ARGUMENT, "slots must be in [1, 64]");
    intp_server* s = new (std::nothrow) intp_server();
    if (!s) return sfail(INTP_ERR_OUT_OF_MEMORY, "out of host memory");
    if (c.memory_budget > 0) s->budget = c.memory_budget;
    if (c.max_batch_points > 0) s->max_batch_points = c.max_batch_points;
    if (const char* tp = std::getenv("INTP_GB300_SERVER_TRACE")) s->trace_path = tp;
    cudaGetDevice(&s->device);
    s->slots.resize(static_cast<size_t>(nslots));
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    const int nsmall = nslots >= 2 ? std::max(1, nslots / 4) : 0;
    for (int i = 0; i < nslots; ++i) {
        Slot& sl = s->slots[static_cast<size_t>(i)];
        sl.small_only = i < nsmall;
        cudaError_t e = cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking, sl.small_only ? greatest : least);
        // tracing times each unit on the device (timing events)
        const unsigned ev_flags = s->trace_path.empty() ? cudaEventDisableTiming : cudaEventDefault;
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, ev_flags);
        if (e == cudaSuccess && !s->trace_path.empty()) e = cudaEventCreateWithFlags(&sl.start, cudaEventDefault);
        if (e != cudaSuccess) {
            delete s;
            return sfail(INTP_ERR_CUDA, std::string("server streams: ") + cudaGetErrorString(e));
        }
    }
    // keep freed pool memory in the pool, and reserve the working set up front
    retain_pool_memory();
    {
        const size_t reserve = static_cast<size_t>(std::min<uint64_t>(s->budget, kPoolReserve));
        cudaStream_t st = s->slots[0].stream;
        void* p = nullptr;
        if (cudaMallocAsync(&p, reserve, st) == cudaSuccess) {
            cudaFreeAsync(p, st);
            cudaStreamSynchronize(st);
        } else {
            cudaGetLastError();  // not fatal: the pool then grows on demand
        }
    }
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return INTP_OK;
}

intp_status intp_server_destroy(intp_server* s) {
    delete s;
    return INTP_OK;
}

intp_status intp_server_submit_build(intp_server* s, const intp_table_desc* desc, const double* values,
                                     int64_t* table_id, int64_t* request_id) {
    if (!s || !desc || !values || !table_id || !request_id) return sfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    if (desc->dim < 1 || desc->dim > INTP_GPU_MAX_DIM) return sfail(INTP_ERR_UNSUPPORTED, "dimension must be in [1, 4]");
    if (desc->channels < 0 || desc->channels > INTP_GPU_MAX_CHANNELS)
        return sfail(INTP_ERR_INVALID_ARGUMENT, "channels must be in [0, 64]");
    Request* r = new (std::nothrow) Request();
    if (!r) return sfail(INTP_ERR_OUT_OF_MEMORY, "out of host memory");
    r->build = true;
    r->desc = *desc;
    for (int d = 0; d < desc->dim; ++d)
        if (desc->coords[d]) {
            const size_t n = static_cast<size_t>(desc->size[d] + (desc->periodic[d] ? 1 : 0));
            r->axis_coords[d].assign(desc->coords[d], desc->coords[d] + n);
            r->desc.coords[d] = r->axis_coords[d].data();
        }
    r->values = values;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> g(s->mu);
        r->id = s->next_request++;
        r->table = s->next_table++;
        Table& tb = s->tables[r->table];
        tb.state = kQueued;
        tb.dim = desc->dim;
        tb.channels = desc->channels > 1 ? desc->channels : 1;
        s->requests[r->id] = r;
        s->pending.push_back(r);
        *table_id = r->table;
        *request_id = r->id;
    }
    s->cv_work.notify_one();
    return INTP_OK;
}

intp_status intp_server_submit_eval(intp_server* s, int64_t table_id, const double* coords, int64_t npts,
                                    const int32_t* derivs, int32_t nderiv, void* out, int32_t out_dtype,
                                    int64_t* request_id) {
    if (!s || !request_id) return sfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    if (npts < 0 || (npts > 0 && (!coords || !out))) return sfail(INTP_ERR_INVALID_ARGUMENT, "null buffer");
    if (out_dtype != INTP_F32 && out_dtype != INTP_F64) return sfail(INTP_ERR_INVALID_ARGUMENT, "unknown output dtype");
    if (derivs && (nderiv < 1 || nderiv > INTP_GPU_MAX_DERIV))
        return sfail(INTP_ERR_INVALID_ARGUMENT, "nderiv must be in [1, 16]");
    Request* r = new (std::nothrow) Request();
    if (!r) return sfail(INTP_ERR_OUT_OF_MEMORY, "out of host memory");
    r->table = table_id;
    r->coords = coords;
    r->npts = npts;
    r->out = out;
    r->out_dtype = out_dtype;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> g(s->mu);
        auto it = s->tables.find(table_id);
        if (it == s->tables.end()) {
            delete r;
            return sfail(INTP_ERR_INVALID_ARGUMENT, "unknown table id");
        }
        if (derivs) {
            r->derivs.assign(derivs, derivs + static_cast<size_t>(nderiv) * it->second.dim);
            r->nderiv = nderiv;
        }
        it->second.refs++;
        r->id = s->next_request++;
        s->requests[r->id] = r;
        s->pending.push_back(r);
        *request_id = r->id;
    }
    s->cv_work.notify_one();
    return INTP_OK;
}

intp_status intp_server_wait(intp_server* s, int64_t request_id, double timeout_s, intp_status* result) {
    if (!s || !result) return sfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end()) return sfail(INTP_ERR_INVALID_ARGUMENT, "unknown or already completed request id");
    Request* r = it->second;
    const auto pred = [r] { return r->done; };
    if (timeout_s < 0) {
        s->cv_done.wait(lock, pred);
    } else if (!s->cv_done.wait_for(lock, std::chrono::duration<double>(timeout_s), pred)) {
        return sfail(INTP_ERR_TIMEOUT, "request still running");
    }
    *result = r->status;
    if (r->status != INTP_OK) set_last_error(r->error);
    s->requests.erase(it);
    delete r;
    return INTP_OK;
}

intp_status intp_server_release(intp_server* s, int64_t table_id) {
    if (!s) return sfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->tables.find(table_id);
    if (it == s->tables.end()) return sfail(INTP_ERR_INVALID_ARGUMENT, "unknown table id");
    Table& tb = it->second;
    tb.release = true;
    if (tb.refs == 0 && tb.state == kResident) s->drop_table(table_id, tb);
    return INTP_OK;
}

intp_status intp_server_table_state(intp_server* s, int64_t table_id, int32_t* state) {
    if (!s || !state) return sfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->tables.find(table_id);
    if (it == s->tables.end()) return sfail(INTP_ERR_INVALID_ARGUMENT, "unknown table id");
    *state = it->second.state;
    return INTP_OK;
}

intp_status intp_server_get_stats(intp_server* s, intp_server_stats* out) {
    if (!s || !out) return sfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> g(s->mu);
    std::memset(out, 0, sizeof *out);
    out->builds_done = static_cast<int64_t>(s->lat_build.size());
    out->evals_done = static_cast<int64_t>(s->lat_eval.size());
    out->failed = s->failed;
    out->evictions = s->evictions;
    out->merged_units = s->merged_units;
    for (auto& kv : s->tables) out->resident_tables += kv.second.state == kResident ? 1 : 0;
    out->resident_bytes = s->resident_bytes;
    out->inflight_bytes = s->inflight_bytes;
    out->points_evaluated = s->points;
    out->build_p50_ms = percentile(s->lat_build, 0.50);
    out->build_p99_ms = percentile(s->lat_build, 0.99);
    out->eval_p50_ms = percentile(s->lat_eval, 0.50);
    out->eval_p99_ms = percentile(s->lat_eval, 0.99);
    std::vector<double> all(s->lat_build);
    all.insert(all.end(), s->lat_eval.begin(), s->lat_eval.end());
    out->all_p50_ms = percentile(all, 0.50);
    out->all_p99_ms = percentile(all, 0.99);
    const double span = ms_since(s->t_reset, s->t_last) / 1e3;
    out->points_per_s = span > 0 ? s->points / span : 0.0;
    return INTP_OK;
}

intp_status intp_server_reset_stats(intp_server* s) {
    if (!s) return sfail(INTP_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> g(s->mu);
    s->lat_build.clear();
    s->lat_eval.clear();
    s->points = 0;
    s->failed = s->evictions = s->merged_units = 0;
    s->t_reset = s->t_last = Clock::now();
    return INTP_OK;
}

}  // extern "C"
