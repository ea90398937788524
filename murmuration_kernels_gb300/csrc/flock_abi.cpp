// C ABI of the GB300 flock step (include/flock_gb300.h): the .flk file,
// the benchmark generator, and the plain / batched / served handles over the
// engine. Every entry point catches engine errors and returns a status code.
#include "../../include/flock_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "flock_engine.h"
#include "flock_params.h"

using flk::Engine;
using flk::Error;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

template <class F>
int guarded(F&& f) {
    try {
        return f();
    } catch (const Error& e) {
        return fail(e.code, e.msg);
    } catch (const std::bad_alloc&) {
        return fail(FLK_ERR_ARG, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(FLK_ERR_ARG, e.what());
    }
}

int check_device(Engine& e) {
    const uint32_t err = e.check_device_error();
    if (err) return fail(FLK_ERR_DEVICE, std::string("device: ") + flk_device_error_text(err));
    return FLK_OK;
}

// ---- .flk file (reference crates/flock-ref/src/state.rs:104-171) ----------
int read_flk(const char* path, float* time, std::vector<float>* words) {
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(FLK_ERR_IO, std::string(path) + ": cannot open");
    uint32_t head[4];
    if (std::fread(head, 4, 4, fp) != 4) {
        std::fclose(fp);
        return fail(FLK_ERR_IO, std::string(path) + ": truncated header");
    }
    if (std::memcmp(head, "FLK1", 4) != 0 || head[2] != (uint32_t)flk::WORDS) {
        std::fclose(fp);
        return fail(FLK_ERR_FORMAT, std::string(path) + ": not a FLK1 file with 15 words per bird");
    }
    std::memcpy(time, &head[3], 4);
    words->resize((size_t)head[1] * flk::WORDS);
    const size_t got = words->empty() ? 0 : std::fread(words->data(), 4, words->size(), fp);
    std::fclose(fp);
    if (got != words->size()) return fail(FLK_ERR_IO, std::string(path) + ": truncated");
    return FLK_OK;
}

int write_flk(const char* path, float time, const float* words, uint32_t n) {
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return fail(FLK_ERR_IO, std::string(path) + ": cannot open for writing");
    uint32_t head[4] = {0x314B4C46u, n, (uint32_t)flk::WORDS, 0u};
    std::memcpy(&head[3], &time, 4);
    bool ok = std::fwrite(head, 4, 4, fp) == 4;
    if (ok && n) ok = std::fwrite(words, 4, (size_t)n * flk::WORDS, fp) == (size_t)n * flk::WORDS;
    ok &= std::fclose(fp) == 0;
    return ok ? FLK_OK : fail(FLK_ERR_IO, std::string(path) + ": write failed");
}

}  // namespace

namespace flk {
// Lets entry points defined in other translation units report through flk_last_error().
__attribute__((visibility("hidden"))) void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace flk

// ---------------------------------------------------------------------------
// plain single flock
// ---------------------------------------------------------------------------
struct flk_flock {
    std::unique_ptr<Engine> eng;
    int id = -1;
    uint32_t n = 0;
};

extern "C" int flk_open_host(int32_t device, uint32_t n, float time, const float* words, flk_flock** out) {
    if (!out || (n && !words)) return fail(FLK_ERR_ARG, "flk_open_host: null pointer");
    *out = nullptr;
    return guarded([&] {
        auto f = std::make_unique<flk_flock>();
        f->eng = std::make_unique<Engine>(device);
        f->id = f->eng->add_flock(n, time, words);
        f->n = n;
        f->eng->sync();
        *out = f.release();
        return FLK_OK;
    });
}

extern "C" int flk_open_file(int32_t device, const char* path, flk_flock** out) {
    if (!path || !out) return fail(FLK_ERR_ARG, "flk_open_file: null pointer");
    float time = 0.f;
    std::vector<float> w;
    int rc = read_flk(path, &time, &w);
    if (rc) return rc;
    return flk_open_host(device, (uint32_t)(w.size() / flk::WORDS), time, w.data(), out);
}

extern "C" int flk_step(flk_flock* f, uint32_t steps) {
    if (!f) return fail(FLK_ERR_ARG, "flk_step: null handle");
    return guarded([&] {
        f->eng->set_remaining({f->id}, {steps});
        f->eng->run(steps);
        f->eng->sync();
        return check_device(*f->eng);
    });
}

extern "C" int flk_step_timed(flk_flock* f, uint32_t steps, uint32_t warmup, flk_pass_times* out) {
    if (!f) return fail(FLK_ERR_ARG, "flk_step_timed: null handle");
    return guarded([&] {
        f->eng->set_remaining({f->id}, {steps});
        flk::PassTimes pt{};
        f->eng->run_timed(steps, warmup, &pt);
        if (out) {
            out->hash_ms = pt.ms[0];
            out->scan_ms = pt.ms[1];
            out->sort_ms = pt.ms[2];
            out->decide_ms = pt.ms[3];
            out->integrate_ms = pt.ms[4];
            out->total_ms = pt.total_ms;
            out->timed_steps = pt.timed_steps;
        }
        return check_device(*f->eng);
    });
}

extern "C" int flk_read_host(flk_flock* f, float* time, float* words) {
    if (!f || (f->n && !words)) return fail(FLK_ERR_ARG, "flk_read_host: null pointer");
    return guarded([&] {
        f->eng->read_flock(f->id, time, words);
        return FLK_OK;
    });
}

extern "C" int flk_write_file(flk_flock* f, const char* path) {
    if (!f || !path) return fail(FLK_ERR_ARG, "flk_write_file: null pointer");
    std::vector<float> w((size_t)f->n * flk::WORDS);
    float time = 0.f;
    int rc = flk_read_host(f, &time, w.data());
    if (rc) return rc;
    return write_flk(path, time, w.data(), f->n);
}

extern "C" int flk_decide_occupancy(flk_flock* f, uint64_t extra_smem, int32_t* blocks_per_sm, int32_t* threads,
                                    int32_t* threads_per_sm, uint64_t* smem_bytes) {
    if (!f) return fail(FLK_ERR_ARG, "flk_decide_occupancy: null handle");
    return guarded([&] {
        flk::LaunchShape s = f->eng->shape();
        s.decide_extra_smem = (size_t)extra_smem;
        f->eng->set_shape(s);  // rejects a reservation no CTA can hold
        int bps = 0, th = 0, tpsm = 0;
        size_t smem = 0;
        f->eng->decide_occupancy(&bps, &th, &smem);
        const cudaError_t e = cudaDeviceGetAttribute(&tpsm, cudaDevAttrMaxThreadsPerMultiProcessor, f->eng->device());
        if (e != cudaSuccess) return fail(FLK_ERR_CUDA, std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
        if (blocks_per_sm) *blocks_per_sm = bps;
        if (threads) *threads = th;
        if (threads_per_sm) *threads_per_sm = tpsm;
        if (smem_bytes) *smem_bytes = smem;
        return FLK_OK;
    });
}

extern "C" const char* flk_device_error_text(uint32_t word) { return flk::device_error_text(word); }

extern "C" int flk_debug_scan_timeout(flk_flock* f, uint32_t skip_tile, uint32_t spin_limit) {
    if (!f) return fail(FLK_ERR_ARG, "flk_debug_scan_timeout: null handle");
    return guarded([&] {
        f->eng->arm_scan_timeout(skip_tile, spin_limit);
        return FLK_OK;
    });
}

extern "C" int flk_size(const flk_flock* f, uint32_t* n, uint32_t* buckets) {
    if (!f) return fail(FLK_ERR_ARG, "flk_size: null handle");
    if (n) *n = f->n;
    if (buckets) *buckets = flk::buckets_for(f->n);
    return FLK_OK;
}

static void copy_debug(const flk::GridDebug& g, uint32_t* keys, uint32_t* offsets, uint32_t* sorted, uint32_t* sets) {
    if (keys && !g.keys.empty()) std::memcpy(keys, g.keys.data(), g.keys.size() * 4);
    if (offsets) std::memcpy(offsets, g.offsets.data(), g.offsets.size() * 4);
    if (sorted && !g.sorted.empty()) std::memcpy(sorted, g.sorted.data(), g.sorted.size() * 4);
    if (sets && !g.sets.empty()) std::memcpy(sets, g.sets.data(), g.sets.size() * 4);
}

extern "C" int flk_step_debug(flk_flock* f, uint32_t* keys, uint32_t* offsets, uint32_t* sorted, uint32_t* sets) {
    if (!f) return fail(FLK_ERR_ARG, "flk_step_debug: null handle");
    return guarded([&] {
        f->eng->set_remaining({f->id}, {1u});
        std::vector<flk::GridDebug> dbg;
        f->eng->step_debug(&dbg);
        if (dbg.size() != 1) return fail(FLK_ERR_ARG, "flk_step_debug: flock not stepped");
        copy_debug(dbg[0], keys, offsets, sorted, sets);
        return check_device(*f->eng);
    });
}

extern "C" int flk_step_f64(flk_flock* f, double* out64, double* report) {
    if (!f) return fail(FLK_ERR_ARG, "flk_step_f64: null handle");
    return guarded([&] {
        f->eng->set_remaining({f->id}, {1u});
        std::vector<std::vector<double>> out;
        std::vector<std::array<double, 4>> rep;
        f->eng->step_f64(&out, &rep);
        if (out.size() != 1) return fail(FLK_ERR_ARG, "flk_step_f64: flock not stepped");
        if (out64 && !out[0].empty()) std::memcpy(out64, out[0].data(), out[0].size() * 8);
        if (report) std::memcpy(report, rep[0].data(), 4 * sizeof(double));
        return check_device(*f->eng);
    });
}

extern "C" int flk_counters(flk_flock* f, uint64_t* due, uint64_t* cand, uint64_t* pairs) {
    if (!f) return fail(FLK_ERR_ARG, "flk_counters: null handle");
    return guarded([&] {
        unsigned long long a, b, c;
        f->eng->counters(&a, &b, &c);
        if (due) *due = a;
        if (cand) *cand = b;
        if (pairs) *pairs = c;
        return FLK_OK;
    });
}

extern "C" int flk_time_steps(flk_flock* f, uint32_t steps, uint64_t flush_bytes, float* ms_per_step) {
    if (!f || (steps && !ms_per_step)) return fail(FLK_ERR_ARG, "flk_time_steps: null pointer");
    if (steps == UINT32_MAX) return fail(FLK_ERR_ARG, "flk_time_steps: too many steps");
    return guarded([&] {
        f->eng->set_remaining({f->id}, {steps + 1});  // the timed steps and one untimed step
        f->eng->time_steps_cold(steps, (size_t)flush_bytes, ms_per_step);
        return check_device(*f->eng);
    });
}

extern "C" void flk_close(flk_flock* f) {
    try {
        delete f;
    } catch (...) {
    }
}

// ---------------------------------------------------------------------------
// batched
// ---------------------------------------------------------------------------
struct flk_batch {
    std::unique_ptr<Engine> eng;
};

extern "C" int flk_batch_create(int32_t device, flk_batch** out) {
    if (!out) return fail(FLK_ERR_ARG, "flk_batch_create: null pointer");
    *out = nullptr;
    return guarded([&] {
        auto b = std::make_unique<flk_batch>();
        b->eng = std::make_unique<Engine>(device);
        *out = b.release();
        return FLK_OK;
    });
}

extern "C" int flk_batch_add(flk_batch* b, uint32_t n, float time, const float* words, int32_t* id) {
    if (!b || !id || (n && !words)) return fail(FLK_ERR_ARG, "flk_batch_add: null pointer");
    return guarded([&] {
        *id = b->eng->add_flock(n, time, words);
        return FLK_OK;
    });
}

extern "C" int flk_batch_remove(flk_batch* b, int32_t id) {
    if (!b) return fail(FLK_ERR_ARG, "flk_batch_remove: null handle");
    return guarded([&] {
        b->eng->remove_flock(id);
        return FLK_OK;
    });
}

extern "C" int flk_batch_step(flk_batch* b, uint32_t steps) {
    if (!b) return fail(FLK_ERR_ARG, "flk_batch_step: null handle");
    return guarded([&] {
        std::vector<int> ids = b->eng->flock_ids();
        b->eng->set_remaining(ids, std::vector<uint32_t>(ids.size(), steps));
        b->eng->run(steps);
        b->eng->sync();
        return check_device(*b->eng);
    });
}

extern "C" int flk_batch_step_each(flk_batch* b, const int32_t* ids, const uint32_t* steps, uint32_t count) {
    if (!b || (count && (!ids || !steps))) return fail(FLK_ERR_ARG, "flk_batch_step_each: null pointer");
    return guarded([&] {
        std::vector<int> v(ids, ids + count);
        std::vector<uint32_t> s(steps, steps + count);
        uint32_t most = 0;
        for (uint32_t k = 0; k < count; ++k) most = std::max(most, steps[k]);
        b->eng->set_remaining(v, s);
        b->eng->run(most);
        b->eng->sync();
        return check_device(*b->eng);
    });
}

extern "C" int flk_batch_read(flk_batch* b, int32_t id, float* time, float* words) {
    if (!b) return fail(FLK_ERR_ARG, "flk_batch_read: null handle");
    return guarded([&] {
        if (!b->eng->has_flock(id)) return fail(FLK_ERR_ID, "flk_batch_read: unknown flock id");
        if (b->eng->flock_size(id) && !words) return fail(FLK_ERR_ARG, "flk_batch_read: null words");
        b->eng->read_flock(id, time, words);
        return FLK_OK;
    });
}

extern "C" int flk_batch_step_debug(flk_batch* b, const int32_t* ids, uint32_t count, uint32_t* keys,
                                    uint32_t* offsets, uint32_t* sorted, uint32_t* sets) {
    if (!b || (count && !ids)) return fail(FLK_ERR_ARG, "flk_batch_step_debug: null pointer");
    return guarded([&] {
        std::vector<int> v(ids, ids + count);
        for (int id : v)
            if (!b->eng->has_flock(id)) return fail(FLK_ERR_ID, "flk_batch_step_debug: unknown flock id");
        b->eng->set_remaining(v, std::vector<uint32_t>(count, 1u));
        std::vector<flk::GridDebug> dbg;
        b->eng->step_debug(&dbg);
        // the engine reports flocks in slot order; map them to the caller's order
        std::vector<int> sorted_ids = v;
        std::sort(sorted_ids.begin(), sorted_ids.end());
        size_t ko = 0, oo = 0, so = 0, zo = 0;
        for (int id : v) {
            const size_t k = (size_t)(std::lower_bound(sorted_ids.begin(), sorted_ids.end(), id) - sorted_ids.begin());
            const flk::GridDebug& g = dbg.at(k);
            copy_debug(g, keys ? keys + ko : nullptr, offsets ? offsets + oo : nullptr, sorted ? sorted + so : nullptr,
                       sets ? sets + zo : nullptr);
            ko += g.keys.size();
            oo += g.offsets.size();
            so += g.sorted.size();
            zo += g.sets.size();
        }
        return check_device(*b->eng);
    });
}

extern "C" int flk_batch_step_f64(flk_batch* b, const int32_t* ids, uint32_t count, double* out64,
                                  double* reports) {
    if (!b || (count && !ids)) return fail(FLK_ERR_ARG, "flk_batch_step_f64: null pointer");
    return guarded([&] {
        std::vector<int> v(ids, ids + count);
        for (int id : v)
            if (!b->eng->has_flock(id)) return fail(FLK_ERR_ID, "flk_batch_step_f64: unknown flock id");
        std::vector<int> sorted_ids = v;
        std::sort(sorted_ids.begin(), sorted_ids.end());
        if (std::adjacent_find(sorted_ids.begin(), sorted_ids.end()) != sorted_ids.end())
            return fail(FLK_ERR_ARG, "flk_batch_step_f64: a flock id is listed twice");
        b->eng->set_remaining(v, std::vector<uint32_t>(count, 1u));
        std::vector<std::vector<double>> out;
        std::vector<std::array<double, 4>> rep;
        b->eng->step_f64(&out, &rep);
        // the engine reports the stepped flocks in slot (= id) order
        if (out.size() != count) return fail(FLK_ERR_ARG, "flk_batch_step_f64: a flock was not stepped");
        size_t o = 0;
        for (uint32_t i = 0; i < count; ++i) {
            const size_t k = (size_t)(std::lower_bound(sorted_ids.begin(), sorted_ids.end(), v[i]) - sorted_ids.begin());
            if (out64 && !out[k].empty()) std::memcpy(out64 + o, out[k].data(), out[k].size() * 8);
            o += out[k].size();
            if (reports) std::memcpy(reports + 4 * (size_t)i, rep[k].data(), 4 * sizeof(double));
        }
        return check_device(*b->eng);
    });
}

extern "C" int flk_batch_tune(flk_batch* b, int32_t stream_bps, int32_t decide_bps, int32_t decide_threads,
                              int32_t graph_chunk) {
    if (!b) return fail(FLK_ERR_ARG, "flk_batch_tune: null handle");
    if (decide_threads && (decide_threads % 32 || decide_threads > 1024 || decide_threads < 32))
        return fail(FLK_ERR_ARG, "flk_batch_tune: decide_threads must be a multiple of 32 in [32, 1024]");
    return guarded([&] {
        flk::LaunchShape s = b->eng->shape();
        if (stream_bps > 0) s.stream_blocks_per_sm = stream_bps;
        if (decide_bps > 0) s.decide_blocks_per_sm = decide_bps;
        if (decide_threads > 0) s.decide_threads = decide_threads;
        if (graph_chunk > 0) s.graph_chunk = graph_chunk;
        b->eng->set_shape(s);
        return FLK_OK;
    });
}

static int set_cell(Engine& e, float cell_m) {
    flk::LaunchShape s = e.shape();
    s.cell = cell_m;
    e.set_shape(s);  // rejects an edge outside [2, 16] m
    return FLK_OK;
}

static int set_decide(Engine& e, int32_t staged) {
    flk::LaunchShape s = e.shape();
    s.decide_kind = staged;
    e.set_shape(s);  // rejects anything but 0 or 1
    return FLK_OK;
}

extern "C" int flk_batch_tune_decide(flk_batch* b, int32_t staged) {
    if (!b) return fail(FLK_ERR_ARG, "flk_batch_tune_decide: null handle");
    return guarded([&] { return set_decide(*b->eng, staged); });
}

extern "C" int flk_tune_decide(flk_flock* f, int32_t staged) {
    if (!f) return fail(FLK_ERR_ARG, "flk_tune_decide: null handle");
    return guarded([&] { return set_decide(*f->eng, staged); });
}

extern "C" int flk_batch_tune_cell(flk_batch* b, float cell_m) {
    if (!b) return fail(FLK_ERR_ARG, "flk_batch_tune_cell: null handle");
    return guarded([&] { return set_cell(*b->eng, cell_m); });
}

extern "C" int flk_tune_cell(flk_flock* f, float cell_m) {
    if (!f) return fail(FLK_ERR_ARG, "flk_tune_cell: null handle");
    return guarded([&] { return set_cell(*f->eng, cell_m); });
}

extern "C" int flk_batch_graph_counts(flk_batch* b, uint64_t* instantiated, uint64_t* updated) {
    if (!b || !instantiated || !updated) return fail(FLK_ERR_ARG, "flk_batch_graph_counts: null pointer");
    b->eng->graph_counts(instantiated, updated);
    return FLK_OK;
}

extern "C" int flk_batch_counters(flk_batch* b, uint64_t* due, uint64_t* cand, uint64_t* pairs) {
    if (!b) return fail(FLK_ERR_ARG, "flk_batch_counters: null handle");
    return guarded([&] {
        unsigned long long a, c, d;
        b->eng->counters(&a, &c, &d);
        if (due) *due = a;
        if (cand) *cand = c;
        if (pairs) *pairs = d;
        return FLK_OK;
    });
}

extern "C" int flk_batch_time_steps(flk_batch* b, uint32_t steps, double* ms) {
    if (!b || !ms) return fail(FLK_ERR_ARG, "flk_batch_time_steps: null pointer");
    return guarded([&] {
        std::vector<int> ids = b->eng->flock_ids();
        b->eng->set_remaining(ids, std::vector<uint32_t>(ids.size(), steps));
        *ms = b->eng->time_run(steps);
        return check_device(*b->eng);
    });
}

extern "C" int flk_batch_step_timed(flk_batch* b, uint32_t steps, uint32_t warmup, flk_pass_times* out) {
    if (!b) return fail(FLK_ERR_ARG, "flk_batch_step_timed: null handle");
    return guarded([&] {
        std::vector<int> ids = b->eng->flock_ids();
        b->eng->set_remaining(ids, std::vector<uint32_t>(ids.size(), steps));
        flk::PassTimes pt{};
        b->eng->run_timed(steps, warmup, &pt);
        if (out) {
            out->hash_ms = pt.ms[0];
            out->scan_ms = pt.ms[1];
            out->sort_ms = pt.ms[2];
            out->decide_ms = pt.ms[3];
            out->integrate_ms = pt.ms[4];
            out->total_ms = pt.total_ms;
            out->timed_steps = pt.timed_steps;
        }
        return check_device(*b->eng);
    });
}

extern "C" void flk_batch_destroy(flk_batch* b) {
    try {
        delete b;
    } catch (...) {
    }
}

// ---------------------------------------------------------------------------
// served: continuous batching
// ---------------------------------------------------------------------------
#define FLK_CUDA_ABI(call)                                                               \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) throw Error{FLK_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)}; \
    } while (0)

namespace {
using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t ticket;
    uint32_t n, steps;
    float time;
    const float* words;
    float* out_words;
    float* out_time;
    size_t bytes;
    Clock::time_point t_submit, t_done;
    int state = 0;  // 0 queued, 1 resident, 2 done, <0 error
    int flock = -1;
    float result_time = 0.f;
    std::vector<float> owned;  // the input state, when the pool holds its own copy (file restore)
};

// A copy of a resident flock's state taken at a chunk boundary.
struct Snapshot {
    std::shared_ptr<Request> r;
    float* words;
    float time = 0.f;
    uint32_t steps_done = 0;
    int state = 0;  // 0 pending, 1 landed, <0 error
};
}  // namespace

struct Retire {
    std::shared_ptr<Request> r;
    cudaEvent_t done;  // recorded when the result has reached the caller's buffer
    float time;
    bool failed;
    std::shared_ptr<Snapshot> snap;  // set: this copy is a snapshot, not the request's result
};

struct flk_pool {
    std::unique_ptr<Engine> eng;
    uint64_t budget = 0;
    uint32_t chunk = 10;
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_retire;
    std::deque<uint64_t> queue;                      // tickets waiting for admission, FIFO
    std::map<uint64_t, std::shared_ptr<Request>> reqs;
    std::vector<std::shared_ptr<Request>> resident;  // admitted, in flight
    std::deque<Retire> retiring;                     // results on their way to the host
    std::vector<std::shared_ptr<Snapshot>> snaps;    // snapshots of resident flocks, waiting for a boundary
    uint64_t next_ticket = 1;
    uint64_t resident_bytes = 0;
    bool stop = false, stop_completer = false;
    flk_pool_stats stats{};
    std::thread worker, completer;
    std::string worker_error;

    void loop();
    void complete_loop();
    std::vector<std::shared_ptr<Request>> take_admissions();
};

// FIFO admission against the memory budget (caller holds no lock).
std::vector<std::shared_ptr<Request>> flk_pool::take_admissions() {
    std::vector<std::shared_ptr<Request>> admit;
    std::lock_guard<std::mutex> lk(mu);
    while (!queue.empty()) {
        auto r = reqs.at(queue.front());
        if (resident_bytes + r->bytes > budget) break;
        resident_bytes += r->bytes;
        queue.pop_front();
        admit.push_back(r);
    }
    return admit;
}

// The device worker. Each turn: admit arrivals (their states start crossing
// the link on the copy stream while the current chunk runs), wait for the
// chunk, hand finished flocks' results to the copy stream, launch the next
// chunk with the new arrivals folded in. Arrivals therefore join at chunk
// boundaries and their uploads and the results' downloads overlap compute.
void flk_pool::loop() {
    try {
        cudaSetDevice(eng->device());
        bool running = false;  // a chunk is in flight on the compute stream
        auto t0 = Clock::now();
        while (true) {
            if (!running) {
                std::unique_lock<std::mutex> lk(mu);
                cv_work.wait(lk, [&] { return stop || !queue.empty() || !resident.empty(); });
                if (stop) return;
            } else {
                std::lock_guard<std::mutex> lk(mu);
                if (stop) return;
            }
            for (auto& r : take_admissions()) {
                r->flock = eng->add_flock_async(r->n, r->time, r->words);
                eng->set_flock_remaining(r->flock, r->steps);
                std::lock_guard<std::mutex> lk(mu);
                r->state = 1;
                resident.push_back(r);
            }
            if (running) {
                eng->sync();
                running = false;
                const uint32_t err = eng->check_device_error();
                std::vector<std::shared_ptr<Request>> live;
                {
                    std::lock_guard<std::mutex> lk(mu);
                    live = resident;
                }
                std::vector<int> ids;
                for (auto& r : live) ids.push_back(r->flock);
                const std::vector<uint32_t> left = eng->remaining_of(ids);
                std::vector<Retire> done;
                // snapshots: packed now, on the compute stream, copied out while the next chunk runs
                std::vector<std::shared_ptr<Snapshot>> snap_now;
                {
                    std::lock_guard<std::mutex> lk(mu);
                    snap_now.swap(snaps);
                }
                for (auto& sn : snap_now) {
                    const auto it = std::find(live.begin(), live.end(), sn->r);
                    Retire x{sn->r, nullptr, 0.f, err != 0, sn};
                    FLK_CUDA_ABI(cudaEventCreateWithFlags(&x.done, cudaEventDisableTiming));
                    if (it == live.end() || err) {  // never for a resident request; fail rather than wait
                        x.failed = true;
                        FLK_CUDA_ABI(cudaEventRecord(x.done, eng->stream()));
                    } else {
                        sn->steps_done = sn->r->steps - left[it - live.begin()];
                        eng->read_flock_async(sn->r->flock, &sn->time, sn->words, x.done);
                    }
                    done.push_back(x);
                }
                for (size_t k = 0; k < live.size(); ++k) {
                    if (left[k] != 0 && !err) continue;
                    Retire x{live[k], nullptr, 0.f, err != 0};
                    FLK_CUDA_ABI(cudaEventCreateWithFlags(&x.done, cudaEventDisableTiming));
                    if (!err) eng->read_flock_async(live[k]->flock, &x.time, live[k]->out_words, x.done);
                    else FLK_CUDA_ABI(cudaEventRecord(x.done, eng->stream()));
                    eng->remove_flock(live[k]->flock);
                    done.push_back(x);
                }
                const auto t1 = Clock::now();
                std::lock_guard<std::mutex> lk(mu);
                stats.busy_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
                stats.chunks += 1;
                for (auto& x : done) {
                    if (!x.snap) {
                        resident_bytes -= x.r->bytes;  // the slot is reusable in stream order
                        resident.erase(std::find(resident.begin(), resident.end(), x.r));
                    }
                    retiring.push_back(x);
                }
                stats.resident_bytes = resident_bytes;
                if (!done.empty()) cv_retire.notify_all();
            }
            bool any;
            {
                std::lock_guard<std::mutex> lk(mu);
                any = !resident.empty();
            }
            if (any) {
                t0 = Clock::now();
                eng->run(chunk);  // launched, not waited for
                running = true;
            }
        }
    } catch (const Error& e) {
        std::lock_guard<std::mutex> lk(mu);
        worker_error = e.msg;
        for (auto& kv : reqs)
            if (kv.second->state == 0 || kv.second->state == 1) kv.second->state = FLK_ERR_CUDA;
        stop = true;
        cv_done.notify_all();
    }
}

// Marks requests done as their results land in the caller's buffers.
void flk_pool::complete_loop() {
    cudaSetDevice(eng->device());
    while (true) {
        Retire x;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_retire.wait(lk, [&] { return stop_completer || !retiring.empty(); });
            if (retiring.empty()) return;
            x = retiring.front();
        }
        const cudaError_t e = cudaEventSynchronize(x.done);
        cudaEventDestroy(x.done);
        std::lock_guard<std::mutex> lk(mu);
        retiring.pop_front();
        if (x.snap) {
            x.snap->state = (x.failed || e != cudaSuccess) ? FLK_ERR_DEVICE : 1;
            cv_done.notify_all();
            continue;
        }
        x.r->t_done = Clock::now();
        x.r->result_time = x.time;
        if (x.r->out_time) *x.r->out_time = x.time;
        if (x.failed || e != cudaSuccess) {
            x.r->state = x.failed ? FLK_ERR_DEVICE : FLK_ERR_CUDA;
        } else {
            x.r->state = 2;
            stats.completed += 1;
            stats.bird_steps += (uint64_t)x.r->n * x.r->steps;
        }
        cv_done.notify_all();
    }
}

extern "C" int flk_pool_create(int32_t device, uint64_t budget_bytes, uint32_t chunk_steps, flk_pool** out) {
    if (!out) return fail(FLK_ERR_ARG, "flk_pool_create: null pointer");
    *out = nullptr;
    return guarded([&] {
        auto p = std::make_unique<flk_pool>();
        p->eng = std::make_unique<Engine>(device);
        p->budget = budget_bytes;
        p->chunk = chunk_steps ? chunk_steps : 10;
        flk::LaunchShape s = p->eng->shape();
        s.graph_chunk = (int)p->chunk;
        p->eng->set_shape(s);
        flk_pool* raw = p.get();
        p->worker = std::thread([raw] { raw->loop(); });
        p->completer = std::thread([raw] { raw->complete_loop(); });
        *out = p.release();
        return FLK_OK;
    });
}

static int pool_submit(flk_pool* p, uint32_t n, float time, const float* words, std::vector<float>* owned,
                       uint32_t steps, float* out_words, float* out_time, uint64_t* ticket) {
    auto r = std::make_shared<Request>();
    if (owned) {
        r->owned.swap(*owned);
        words = r->owned.data();
    }
    r->n = n;
    r->steps = steps;
    r->time = time;
    r->words = words;
    r->out_words = out_words;
    r->out_time = out_time;
    r->bytes = Engine::bytes_for(n);
    r->t_submit = Clock::now();
    std::lock_guard<std::mutex> lk(p->mu);
    if (p->stop) return fail(FLK_ERR_CUDA, "flk_pool_submit: pool worker stopped: " + p->worker_error);
    p->stats.submitted += 1;
    if (r->bytes > p->budget) {
        p->stats.rejected += 1;
        return fail(FLK_ERR_BUDGET, "flk_pool_submit: flock of " + std::to_string(n) + " birds exceeds the budget");
    }
    r->ticket = p->next_ticket++;
    if (steps == 0) {  // nothing to simulate: complete immediately with the input state
        if (n && out_words != words) std::memcpy(out_words, words, (size_t)n * flk::WORDS * 4);
        if (out_time) *out_time = time;
        r->result_time = time;
        r->state = 2;
        r->t_done = r->t_submit;
        p->stats.completed += 1;
        p->reqs[r->ticket] = r;
        *ticket = r->ticket;
        return FLK_OK;
    }
    p->reqs[r->ticket] = r;
    p->queue.push_back(r->ticket);
    *ticket = r->ticket;
    p->cv_work.notify_one();
    return FLK_OK;
}

extern "C" int flk_pool_submit(flk_pool* p, uint32_t n, float time, const float* words, uint32_t steps,
                               float* out_words, float* out_time, uint64_t* ticket) {
    if (!p || !ticket || (n && (!words || !out_words))) return fail(FLK_ERR_ARG, "flk_pool_submit: null pointer");
    return pool_submit(p, n, time, words, nullptr, steps, out_words, out_time, ticket);
}

extern "C" int flk_pool_submit_file(flk_pool* p, const char* path, uint32_t steps, float* out_words,
                                    uint32_t out_capacity, float* out_time, uint64_t* ticket, uint32_t* n_out) {
    if (!p || !path || !ticket) return fail(FLK_ERR_ARG, "flk_pool_submit_file: null pointer");
    float time = 0.f;
    std::vector<float> w;
    const int rc = read_flk(path, &time, &w);
    if (rc != FLK_OK) return rc;
    const uint32_t n = (uint32_t)(w.size() / flk::WORDS);
    if (n_out) *n_out = n;
    if (n > out_capacity) return fail(FLK_ERR_CAPACITY, "flk_pool_submit_file: " + std::to_string(n) +
                                                           " birds do not fit the result buffer");
    if (n && !out_words) return fail(FLK_ERR_ARG, "flk_pool_submit_file: null result buffer");
    return pool_submit(p, n, time, w.data(), &w, steps, out_words, out_time, ticket);
}

extern "C" int flk_pool_snapshot(flk_pool* p, uint64_t ticket, float* words, float* time, uint32_t* steps_done,
                                 const char* path) {
    if (!p) return fail(FLK_ERR_ARG, "flk_pool_snapshot: null handle");
    std::unique_lock<std::mutex> lk(p->mu);
    auto it = p->reqs.find(ticket);
    if (it == p->reqs.end()) return fail(FLK_ERR_ID, "flk_pool_snapshot: unknown ticket");
    auto r = it->second;
    if (r->n && !words) return fail(FLK_ERR_ARG, "flk_pool_snapshot: null words");
    if (r->state == 1 && std::find(p->resident.begin(), p->resident.end(), r) == p->resident.end())
        p->cv_done.wait(lk, [&] { return r->state != 1 || p->stop; });  // retiring: its result is landing
    if (r->state < 0) return fail(r->state, "flk_pool_snapshot: request failed: " + p->worker_error);
    if (r->state == 1 && p->stop) return fail(FLK_ERR_CUDA, "flk_pool_snapshot: pool stopped");
    float t = 0.f;
    uint32_t k = 0;
    const size_t bytes = (size_t)r->n * flk::WORDS * 4;
    if (r->state == 0) {  // still queued: its input state
        if (bytes) std::memcpy(words, r->words, bytes);
        t = r->time;
    } else if (r->state == 2) {  // finished: its result
        if (bytes) std::memcpy(words, r->out_words, bytes);
        t = r->result_time;
        k = r->steps;
    } else {  // resident: taken at the next chunk boundary while the others keep running
        auto sn = std::make_shared<Snapshot>();
        sn->r = r;
        sn->words = words;
        p->snaps.push_back(sn);
        p->cv_work.notify_one();
        p->cv_done.wait(lk, [&] { return sn->state != 0 || p->stop; });
        if (sn->state != 1) return fail(sn->state ? sn->state : FLK_ERR_CUDA, "flk_pool_snapshot: copy failed");
        t = sn->time;
        k = sn->steps_done;
    }
    lk.unlock();
    if (time) *time = t;
    if (steps_done) *steps_done = k;
    return path ? write_flk(path, t, words, r->n) : FLK_OK;
}

extern "C" int flk_pool_error_report(flk_pool* p, uint64_t ticket, double* out64, double* report,
                                     uint32_t* steps_done) {
    if (!p) return fail(FLK_ERR_ARG, "flk_pool_error_report: null handle");
    uint32_t n = 0;
    {
        std::lock_guard<std::mutex> lk(p->mu);
        auto it = p->reqs.find(ticket);
        if (it == p->reqs.end()) return fail(FLK_ERR_ID, "flk_pool_error_report: unknown ticket");
        n = it->second->n;
    }
    std::vector<float> words((size_t)n * flk::WORDS);
    float t = 0.f;
    int rc = flk_pool_snapshot(p, ticket, words.data(), &t, steps_done, nullptr);
    if (rc) return rc;
    // the evaluation runs on a private copy on the pool's device, beside the
    // worker's stream: the served flock is neither paused beyond the
    // snapshot's chunk boundary nor advanced
    flk_flock* f = nullptr;
    rc = flk_open_host(p->eng->device(), n, t, words.data(), &f);
    if (rc) return rc;
    rc = flk_step_f64(f, out64, report);
    flk_close(f);
    return rc;
}

extern "C" int flk_pool_poll(flk_pool* p, uint64_t ticket, int32_t* state) {
    if (!p || !state) return fail(FLK_ERR_ARG, "flk_pool_poll: null pointer");
    std::lock_guard<std::mutex> lk(p->mu);
    auto it = p->reqs.find(ticket);
    if (it == p->reqs.end()) return fail(FLK_ERR_ID, "flk_pool_poll: unknown ticket");
    *state = it->second->state;
    return FLK_OK;
}

extern "C" int flk_pool_wait(flk_pool* p, uint64_t ticket, double* latency_ms) {
    if (!p) return fail(FLK_ERR_ARG, "flk_pool_wait: null handle");
    std::unique_lock<std::mutex> lk(p->mu);
    auto it = p->reqs.find(ticket);
    if (it == p->reqs.end()) return fail(FLK_ERR_ID, "flk_pool_wait: unknown ticket");
    auto r = it->second;
    p->cv_done.wait(lk, [&] { return r->state == 2 || r->state < 0; });
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    if (r->state < 0) return fail(r->state, "flk_pool_wait: request failed: " + p->worker_error);
    return FLK_OK;
}

extern "C" int flk_pool_stats_get(flk_pool* p, flk_pool_stats* out) {
    if (!p || !out) return fail(FLK_ERR_ARG, "flk_pool_stats_get: null pointer");
    std::lock_guard<std::mutex> lk(p->mu);
    *out = p->stats;
    return FLK_OK;
}

extern "C" void flk_pool_destroy(flk_pool* p) {
    if (!p) return;
    {
        std::lock_guard<std::mutex> lk(p->mu);
        p->stop = true;
    }
    p->cv_work.notify_all();
    if (p->worker.joinable()) p->worker.join();
    {
        // results already on their way still land before the pool goes
        std::lock_guard<std::mutex> lk(p->mu);
        p->stop_completer = true;
    }
    p->cv_retire.notify_all();
    if (p->completer.joinable()) p->completer.join();
    try {
        delete p;
    } catch (...) {
    }
}

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
extern "C" const char* flk_last_error(void) { return g_last_error.c_str(); }

extern "C" uint32_t flk_buckets_for(uint32_t n) { return flk::buckets_for(n); }

extern "C" int flk_file_info(const char* path, uint32_t* n, float* time) {
    if (!path) return fail(FLK_ERR_ARG, "flk_file_info: null path");
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(FLK_ERR_IO, std::string(path) + ": cannot open");
    uint32_t head[4];
    const bool got = std::fread(head, 4, 4, fp) == 4;
    std::fclose(fp);
    if (!got) return fail(FLK_ERR_IO, std::string(path) + ": truncated header");
    if (std::memcmp(head, "FLK1", 4) != 0 || head[2] != (uint32_t)flk::WORDS)
        return fail(FLK_ERR_FORMAT, std::string(path) + ": not a FLK1 file with 15 words per bird");
    if (n) *n = head[1];
    if (time) std::memcpy(time, &head[3], 4);
    return FLK_OK;
}

// SplitMix64 scatter (reference crates/flock-ref/src/state.rs:58-101): per
// bird, 3 position draws, 3 jitter draws, 1 decision-phase draw.
extern "C" int flk_generate(uint32_t n, uint64_t seed, float* words) {
    if (n && !words) return fail(FLK_ERR_ARG, "flk_generate: null words");
    uint64_t s = seed;
    auto next = [&s]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    auto unit = [&]() { return (float)(next() >> 40) / (float)(1ull << 24); };
    const float side = std::cbrt((float)n / flk::DENSITY);
    for (uint32_t i = 0; i < n; ++i) {
        const float ox = (unit() - 0.5f) * side;
        const float oy = (unit() - 0.5f) * side;
        const float oz = (unit() - 0.5f) * side;
        const float jx = (unit() - 0.5f) * 0.05f;
        const float jy = (unit() - 0.5f) * 0.05f;
        const float jz = (unit() - 0.5f) * 0.05f;
        const float vx = 1.0f + jx, vy = 0.0f + jy, vz = 0.0f + jz;
        const float inv = 1.0f / std::sqrt(vx * vx + vy * vy + vz * vz);
        float* w = words + (size_t)i * flk::WORDS;
        w[0] = 0.0f + ox;
        w[1] = 0.0f + oy;
        w[2] = flk::Z0 + oz;
        w[3] = (vx * inv) * flk::V0;
        w[4] = (vy * inv) * flk::V0;
        w[5] = (vz * inv) * flk::V0;
        w[6] = 0.f;
        w[7] = 0.f;
        w[8] = flk::START_RADIUS;
        w[9] = w[10] = w[11] = 0.f;
        w[12] = unit() * flk::DU;
        const uint32_t zero = 0;
        std::memcpy(&w[13], &zero, 4);
        w[14] = 0.f;
    }
    return FLK_OK;
}

extern "C" int flk_params(float* out, int32_t cap) {
    using namespace flk;
    const float v[28] = {DT,    DU,      V0,    MASS,        CL_CD,     G,         L0,      D0,       TAU,     TAU_ROLL,
                         MAX_ROLL_RATE, MAX_BANK, V_MIN, V_MAX, N_C, R_MAX, RADIUS_LERP, R_H, SIGMA, W_SEP,
                         W_ALIGN, W_COH, BLIND_COS, W_ROOST_V, H_ROOST_V, Z0, GRID_CELL, RADIUS_EXP};
    const int k = std::min<int32_t>(cap, 28);
    if (out && k > 0) std::memcpy(out, v, (size_t)k * 4);
    return k;
}

extern "C" uint64_t flk_bytes_for(uint32_t n) { return Engine::bytes_for(n); }

extern "C" int flk_kernels_per_step(void) { return Engine::kernels_per_step(); }

extern "C" int flk_pin(void* ptr, uint64_t bytes) {
    if (!ptr || !bytes) return fail(FLK_ERR_ARG, "flk_pin: null pointer or zero size");
    const cudaError_t e = cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault);
    if (e != cudaSuccess) return fail(FLK_ERR_CUDA, std::string("cudaHostRegister: ") + cudaGetErrorString(e));
    return FLK_OK;
}

extern "C" int flk_unpin(void* ptr) {
    if (!ptr) return fail(FLK_ERR_ARG, "flk_unpin: null pointer");
    const cudaError_t e = cudaHostUnregister(ptr);
    if (e != cudaSuccess) return fail(FLK_ERR_CUDA, std::string("cudaHostUnregister: ") + cudaGetErrorString(e));
    return FLK_OK;
}
