// GB300 (sm_103a) kernels and host engine for the starling-flock step.
//
// One step (reference order, crates/flock-ref/src/model.rs:182-200 and
// cuda/flock.cu:453-470): time += DT; rebuild the cell grid from the current
// positions; every bird with time >= next_decision decides from a snapshot;
// every bird integrates. The passes here:
//
//   k_hash_count  cell key per bird + bucket histogram with warp-aggregated
//                 atomics (one per run of adjacent lanes with one bucket);
//                 records each bird's arrival rank
//                 and, in grid-reporting steps, appends first-seen buckets to
//                 an occupied-bucket list (one atomic per CTA iteration).
//                 Production steps bucket cells by a lattice index,
//                 grid-reporting steps by the reference's hash.
//   k_place       production steps: lists the occupied buckets in lattice
//                 order from the histogram and gives each its run start from
//                 a per-flock cursor (one atomic per warp).
//   k_scan        grid-reporting steps: single-pass decoupled look-back
//                 exclusive scan of the histogram into the canonical dense
//                 offsets (buckets+1 entries). Bounded waits.
//   k_scatter     bird -> slot in its bucket's run (arrival order).
//   k_segsort     one warp per occupied bucket (contiguous ranges of them per
//                 warp) sorts its run by bird index (the canonical stable
//                 order) and moves those birds' state into the other of the
//                 flock's two state buffers in that order; it also writes each
//                 bird's unit heading and stages the deciding-bird records.
//   k_decide      one warp per deciding bird, one 1024-thread CTA per SM: the
//                 2R neighbourhood's buckets (deduplicated with __match_any_sync
//                 in grid-reporting steps) are swept as one packed sequence of
//                 candidates, hits are queued and processed on full warps,
//                 and a reduce-scatter of shuffles sums them.
//   k_integrate   banked flight, streaming float4 over the reordered buffer;
//                 its last block advances the flock clocks, makes the
//                 reordered buffer current and resets the step counters.
//
// Exactness: the file is compiled with -fmad=false, and the expressions that
// decide set membership use explicit round-to-nearest intrinsics, so cell
// keys, the sorted order and all four neighbour sets equal the CPU oracle's
// bit for bit. Sums run in lane order instead of bird order, so forces agree
// to rounding (about 1e-7 relative), not bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>

#include "flock_engine.h"
#include "flock_params.h"
#include "k_decide.cuh"
#include "k_decide_staged.cuh"
#include "k_fp64.cuh"
#include "k_grid.cuh"
#include "k_integrate.cuh"

namespace flk {

#define FLK_CUDA(call)                                                                                    \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) {                                                                          \
            throw Error{-3, std::string(#call) + ": " + cudaGetErrorString(e_)};                          \
        }                                                                                                 \
    } while (0)

const char* device_error_text(uint32_t word) {
    switch (word) {
        case DEV_OK: return "no device error";
        case DEV_SCAN_TIMEOUT: return "a scan look-back wait gave up (error word 1)";
        case DEV_BAD_RANGE: return "a bucket range or slot fell outside its array and was skipped (error word 2)";
        case DEV_STAGE_TIMEOUT: return "a staged decide's bulk copies did not land in time (error word 3)";
        default: return "unknown device error word";
    }
}

uint32_t buckets_for(uint32_t n) {
    uint64_t want = 1;
    while (want < (uint64_t)n * 2) want <<= 1;
    return (uint32_t)std::min<uint64_t>(std::max<uint64_t>(want, 1u << 16), 1u << 22);
}

// ---------------------------------------------------------------------------
// host engine
// ---------------------------------------------------------------------------
// Device memory cache shared by every engine of the process, per device.
// cudaMalloc of the large arrays and cudaFree (which synchronises the whole
// device) cost more than a short run of steps, so an engine's blocks go back
// to the cache when it releases them (after its streams have finished with
// them) and the next engine that asks for a block of the same rounded size
// on that device takes it. At most CACHE_CAP bytes stay cached per device;
// beyond that, blocks are freed.
namespace {
constexpr int CACHE_DEVICES = 64;
constexpr size_t CACHE_CAP = 16ull << 30;
struct DevCache {
    std::mutex mu;
    std::multimap<size_t, void*> free_blocks;  // rounded size -> block
    std::map<void*, size_t> sizes;             // every block handed out: its rounded size
    size_t cached = 0;
};
DevCache g_cache[CACHE_DEVICES];

size_t round_bytes(size_t b) {
    const size_t g = b <= (1u << 20) ? 4096 : (2u << 20);
    return (b + g - 1) / g * g;
}

void* cache_alloc(int dev, size_t bytes) {
    const size_t rb = round_bytes(std::max<size_t>(bytes, 1));
    DevCache& c = g_cache[dev % CACHE_DEVICES];
    {
        std::lock_guard<std::mutex> lk(c.mu);
        auto it = c.free_blocks.find(rb);
        if (it != c.free_blocks.end()) {
            void* p = it->second;
            c.free_blocks.erase(it);
            c.cached -= rb;
            return p;
        }
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, rb);
    if (e == cudaErrorMemoryAllocation) {
        (void)cudaGetLastError();
        // give the cached blocks back and try once more
        std::lock_guard<std::mutex> lk(c.mu);
        for (auto& kv : c.free_blocks) {
            cudaFree(kv.second);
            c.sizes.erase(kv.second);
        }
        c.free_blocks.clear();
        c.cached = 0;
        e = cudaMalloc(&p, rb);
    }
    if (e != cudaSuccess) throw Error{-3, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
    std::lock_guard<std::mutex> lk(c.mu);
    c.sizes[p] = rb;
    return p;
}

// The caller guarantees that no work in flight uses p.
void cache_free(int dev, void* p) {
    if (!p) return;
    DevCache& c = g_cache[dev % CACHE_DEVICES];
    std::lock_guard<std::mutex> lk(c.mu);
    auto it = c.sizes.find(p);
    if (it == c.sizes.end()) return;  // never for a block from cache_alloc
    const size_t rb = it->second;
    if (c.cached + rb > CACHE_CAP) {
        cudaFree(p);
        c.sizes.erase(it);
        return;
    }
    c.free_blocks.emplace(rb, p);
    c.cached += rb;
}

// Per device, set up once for the process: the radius factor table
// (params.rs:61-65 evaluated with the host libm, 65,536 powf calls) and the
// streaming kernels' resident CTAs per SM.
struct DevStatic {
    std::once_flag once;
    float* radius_table = nullptr;
    int fit[10] = {};
};
DevStatic g_static[CACHE_DEVICES];
}  // namespace

template <class T>
T* Engine::dalloc(size_t n, size_t* acct) {
    if (n == 0) n = 1;
    void* p = cache_alloc(device_, n * sizeof(T));
    *acct += n * sizeof(T);
    return static_cast<T*>(p);
}
template <class T>
void Engine::dfree(T*& p) {
    if (!p) return;
    // the engine's queued work may still use the block: let it finish first
    cudaStreamSynchronize(stream_);
    cudaStreamSynchronize(copy_);
    cache_free(device_, p);
    p = nullptr;
}

Engine::Engine(int device) {
    if (device < 0) FLK_CUDA(cudaGetDevice(&device));
    device_ = device;
    FLK_CUDA(cudaSetDevice(device_));
    FLK_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, device_));
    FLK_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    FLK_CUDA(cudaStreamCreateWithFlags(&copy_, cudaStreamNonBlocking));
    ctl_ = dalloc<StepCtl>(1, &dev_bytes_);
    StepCtl c{};
    c.epoch = 1;
    FLK_CUDA(cudaMemcpyAsync(ctl_, &c, sizeof c, cudaMemcpyHostToDevice, stream_));
    DevStatic& ds = g_static[device_ % CACHE_DEVICES];
    std::call_once(ds.once, [&] {
        std::vector<float> tab(RADIUS_TABLE);
        for (int n = 0; n < RADIUS_TABLE; ++n) {
            const float nn = (float)(n > 1 ? n : 1);
            tab[n] = powf(N_C / nn, RADIUS_EXP);
        }
        FLK_CUDA(cudaMalloc(&ds.radius_table, RADIUS_TABLE * sizeof(float)));  // held for the process
        FLK_CUDA(cudaMemcpy(ds.radius_table, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice));
        auto fit = [](auto kernel) {
            int n = 0;
            FLK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, 256, 0));
            return std::max(1, n);
        };
        const int f[10] = {fit(k_hash_count<false>), fit(k_hash_count<true>), fit(k_place),     fit(k_scatter),
                           fit(k_segsort),           fit(k_integrate<false>), fit(k_integrate<true>),
                           fit(k_decide_f64),        fit(k_integrate_f64),  fit(k_compare_f64)};
        std::copy(f, f + 10, ds.fit);
    });
    if (!ds.radius_table) throw Error{-3, "radius table set-up failed on this device"};
    radius_table_ = ds.radius_table;
    FLK_CUDA(cudaStreamSynchronize(stream_));
    set_shape(shape_);  // decide's shared memory may exceed the default 48 KB per CTA
}

Engine::~Engine() {
    cudaSetDevice(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    if (copy_) cudaStreamSynchronize(copy_);
    destroy_graphs();
    dfree(ar_.A); dfree(ar_.B); dfree(ar_.C); dfree(ar_.D); dfree(ar_.id);
    dfree(table_d_);
    dfree(key_); dfree(arrival_); dfree(tmp_); dfree(occ_); dfree(occ2_); dfree(due_);
    dfree(counts2_);
    dfree(sfwd_); dfree(counts_); dfree(offsets_); dfree(status_); dfree(sets_); dfree(slabs_);
    dfree(ctl_); dfree(staging_);
    dfree(dec64_); dfree(out64_); dfree(active_); dfree(err64_);
    if (copy_) cudaStreamDestroy(copy_);
    if (stream_) cudaStreamDestroy(stream_);
}

// Marks the captured chunk as out of date (sizes, pointers or launch shapes
// changed); the next ensure_graph recaptures it and updates the executable
// graph in place.
void Engine::free_graphs() { graph_stale_ = true; }

void Engine::destroy_graphs() {
    if (graph_) cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
    graph_steps_ = 0;
    graph_stale_ = false;
}

size_t Engine::bytes_for(uint32_t n) {
    // state 2 x 68 B (two buffers) + scratch (key, arrival, two occupied lists
    // 4 B each; tmp 8 B; due record 48 B; heading 16 B) + buckets (two
    // histograms, offsets, slab boundaries 4 B each + status/4096; about one
    // bucket per bird)
    const size_t b = production_buckets(n);
    return (size_t)n * (136 + 88) + b * 16 + (b / SCAN_TILE) * 8 + 256;
}

// staged positions a k_decide_staged CTA holds
static constexpr uint32_t STAGE_CAP = 4096;

size_t Engine::decide_smem(bool sets) const {
    const int w = shape_.decide_threads / 32;
    if (!sets && shape_.decide_kind == 1) return staged_smem_bytes(w, STAGE_CAP) + shape_.decide_extra_smem;
    return (size_t)w * (sets ? decide_smem_per_warp<true>() : decide_smem_per_warp<false>()) +
           shape_.decide_extra_smem;
}

void Engine::decide_occupancy(int* blocks_per_sm, int* threads, size_t* smem_bytes) const {
    const size_t smem = decide_smem(false);
    int n = 0;
    if (shape_.decide_kind == 1)
        FLK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_decide_staged, shape_.decide_threads, smem));
    else
        FLK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_decide<false>, shape_.decide_threads, smem));
    *blocks_per_sm = n;
    *threads = shape_.decide_threads;
    *smem_bytes = smem;
}

void Engine::set_shape(const LaunchShape& s) {
    int optin = 0;
    FLK_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_));
    const size_t w = (size_t)(s.decide_threads / 32);
    if (s.decide_kind != 0 && s.decide_kind != 1) throw Error{-1, "decide kind must be 0 (direct) or 1 (staged)"};
    const size_t need = std::max({w * decide_smem_per_warp<false>(), w * decide_smem_per_warp<true>(),
                                  s.decide_kind == 1 ? staged_smem_bytes((int)w, STAGE_CAP) : (size_t)0}) +
                        s.decide_extra_smem;
    if (need > (size_t)optin)
        throw Error{-1, "decide would need " + std::to_string(need) + " B of shared memory per CTA, above the " +
                            std::to_string(optin) + " B a CTA may have"};
    if (!(s.cell >= 2.0f && s.cell <= 16.0f)) throw Error{-1, "production cell edge must lie in [2, 16] m"};
    shape_ = s;
    // decide's dynamic shared memory grows with its CTA size; allow past 48 KB
    FLK_CUDA(cudaFuncSetAttribute(k_decide<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)decide_smem(false)));
    FLK_CUDA(cudaFuncSetAttribute(k_decide<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)decide_smem(true)));
    if (s.decide_kind == 1)
        FLK_CUDA(cudaFuncSetAttribute(k_decide_staged, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)decide_smem(false)));
    // the streaming kernels' resident CTAs per SM, queried once per device
    const int* f = g_static[device_ % CACHE_DEVICES].fit;
    fit_.hash[0] = f[0];
    fit_.hash[1] = f[1];
    fit_.place = f[2];
    fit_.scatter = f[3];
    fit_.segsort = f[4];
    fit_.integrate[0] = f[5];
    fit_.integrate[1] = f[6];
    fit_.decide_f64 = f[7];
    fit_.integrate_f64 = f[8];
    fit_.compare_f64 = f[9];
    free_graphs();
}

void Engine::ensure_arena(uint32_t need) {
    if (need <= cap_) return;
    // both buffers of a field share one allocation indexed by 32-bit slots
    if (need >= (1u << 31)) throw Error{-5, "arena above 2^31 birds"};
    uint32_t ncap = std::max<uint32_t>(need, cap_ ? cap_ + cap_ / 2 : need);
    ncap = std::min<uint32_t>(ncap, (1u << 31) - 1);
    size_t acct = 0;
    Arena na{};
    na.cap = ncap;
    na.A = dalloc<float4>((size_t)ncap * 2, &acct);
    na.B = dalloc<float4>((size_t)ncap * 2, &acct);
    na.C = dalloc<float4>((size_t)ncap * 2, &acct);
    na.D = dalloc<float4>((size_t)ncap * 2, &acct);
    na.id = dalloc<uint32_t>((size_t)ncap * 2, &acct);
    if (used_) {
        for (size_t p = 0; p < 2; ++p) {
            const size_t o = p * cap_, n = p * ncap;
            FLK_CUDA(cudaMemcpyAsync(na.A + n, ar_.A + o, (size_t)used_ * 16, cudaMemcpyDeviceToDevice, stream_));
            FLK_CUDA(cudaMemcpyAsync(na.B + n, ar_.B + o, (size_t)used_ * 16, cudaMemcpyDeviceToDevice, stream_));
            FLK_CUDA(cudaMemcpyAsync(na.C + n, ar_.C + o, (size_t)used_ * 16, cudaMemcpyDeviceToDevice, stream_));
            FLK_CUDA(cudaMemcpyAsync(na.D + n, ar_.D + o, (size_t)used_ * 16, cudaMemcpyDeviceToDevice, stream_));
            FLK_CUDA(cudaMemcpyAsync(na.id + n, ar_.id + o, (size_t)used_ * 4, cudaMemcpyDeviceToDevice, stream_));
        }
        FLK_CUDA(cudaStreamSynchronize(stream_));
    }
    dev_bytes_ -= (size_t)cap_ * 136;
    dfree(ar_.A); dfree(ar_.B); dfree(ar_.C); dfree(ar_.D); dfree(ar_.id);
    ar_ = na;
    dev_bytes_ += acct;
    cap_ = ncap;
    free_graphs();
}

int Engine::add_flock(uint32_t n, float time, const float* words) {
    FLK_CUDA(cudaSetDevice(device_));
    // first-fit into a hole, else append
    uint32_t sbase = used_;
    bool from_hole = false;
    for (auto& h : free_ranges_) {
        if (h.second >= n) {
            sbase = h.first;
            h.first += n;
            h.second -= n;
            from_hole = true;
            break;
        }
    }
    if (!from_hole) {
        ensure_arena(used_ + n);
        used_ += n;
    }
    free_ranges_.erase(std::remove_if(free_ranges_.begin(), free_ranges_.end(),
                                      [](const std::pair<uint32_t, uint32_t>& h) { return h.second == 0; }),
                       free_ranges_.end());
    if (n) {
        const size_t bytes = (size_t)n * WORDS * 4;
        if (bytes > staging_cap_) {
            dev_bytes_ -= staging_cap_;
            dfree(staging_);
            staging_ = dalloc<float>((size_t)n * WORDS, &dev_bytes_);
            staging_cap_ = bytes;
        }
        FLK_CUDA(cudaMemcpyAsync(staging_, words, bytes, cudaMemcpyHostToDevice, stream_));
        const int blocks = std::min<uint32_t>((n + 255) / 256, (uint32_t)num_sms_ * 8);
        k_unpack<<<blocks, 256, 0, stream_>>>(staging_, n, sbase, ar_);  // buffer 0
        FLK_CUDA(cudaGetLastError());
    }
    Slot s;
    s.n = n;
    s.sbase = sbase;
    s.buckets = buckets_for(n);
    s.remaining = 0;
    s.time = time;
    s.live = true;
    int id = -1;
    for (size_t k = 0; k < slots_.size(); ++k)
        if (!slots_[k].live) { id = (int)k; break; }
    if (id < 0) {
        id = (int)slots_.size();
        slots_.push_back(s);
    } else {
        slots_[id] = s;
    }
    return id;
}

bool Engine::has_flock(int id) const { return id >= 0 && id < (int)slots_.size() && slots_[id].live; }
uint32_t Engine::flock_size(int id) const { return has_flock(id) ? slots_[id].n : 0; }
std::vector<int> Engine::flock_ids() const {
    std::vector<int> ids;
    for (size_t k = 0; k < slots_.size(); ++k)
        if (slots_[k].live) ids.push_back((int)k);
    return ids;
}

void Engine::sync_times() {
    // The device table holds the live clocks and countdowns once steps have
    // run; until then the host copy is authoritative (it may hold step counts
    // set since the last run that the device has not seen yet).
    if (!device_ahead_ || table_h_.empty() || !table_d_) return;
    device_ahead_ = false;
    std::vector<FlockDesc> t(table_h_.size());
    FLK_CUDA(cudaMemcpyAsync(t.data(), table_d_, t.size() * sizeof(FlockDesc), cudaMemcpyDeviceToHost, stream_));
    FLK_CUDA(cudaStreamSynchronize(stream_));
    for (size_t k = 0; k < t.size(); ++k) {
        if (table_ids_[k] < 0) continue;  // removed since the table was built
        Slot& s = slots_[table_ids_[k]];
        s.time = t[k].time;
        s.remaining = t[k].remaining;
        s.parity = t[k].parity;
    }
    table_h_ = t;
}

void Engine::remove_flock(int id) {
    if (!has_flock(id)) throw Error{-4, "unknown flock id"};
    sync_times();
    // the slot id may be reused before the table is rebuilt: detach it
    for (int& t : table_ids_)
        if (t == id) t = -1;
    Slot& s = slots_[id];
    s.live = false;
    if (s.n) {
        free_ranges_.push_back({s.sbase, s.n});
        std::sort(free_ranges_.begin(), free_ranges_.end());
        std::vector<std::pair<uint32_t, uint32_t>> merged;
        for (auto& h : free_ranges_) {
            if (!merged.empty() && merged.back().first + merged.back().second == h.first) merged.back().second += h.second;
            else merged.push_back(h);
        }
        // a hole at the end of the arena returns to the tail
        if (!merged.empty() && merged.back().first + merged.back().second == used_) {
            used_ = merged.back().first;
            merged.pop_back();
        }
        free_ranges_ = merged;
    }
    table_dirty_ = true;
}

float Engine::flock_time(int id) {
    if (!has_flock(id)) throw Error{-4, "unknown flock id"};
    sync_times();
    return slots_[id].time;
}

int Engine::add_flock_async(uint32_t n, float time, const float* words) {
    FLK_CUDA(cudaSetDevice(device_));
    // the state crosses the link on the copy stream while the compute stream
    // keeps running; a stream-ordered staging buffer is unpacked once it lands
    float* stage = nullptr;
    cudaEvent_t landed = nullptr;
    if (n) {
        const size_t bytes = (size_t)n * WORDS * 4;
        FLK_CUDA(cudaMallocAsync((void**)&stage, bytes, copy_));
        FLK_CUDA(cudaMemcpyAsync(stage, words, bytes, cudaMemcpyHostToDevice, copy_));
        FLK_CUDA(cudaEventCreateWithFlags(&landed, cudaEventDisableTiming));
        FLK_CUDA(cudaEventRecord(landed, copy_));
    }
    const int id = add_flock(0, time, nullptr);  // reserves the slot; its state follows
    if (n) {
        Slot& s = slots_[id];
        // move the empty reservation to a real range of n birds
        uint32_t sbase = used_;
        bool from_hole = false;
        for (auto& h : free_ranges_) {
            if (h.second >= n) {
                sbase = h.first;
                h.first += n;
                h.second -= n;
                from_hole = true;
                break;
            }
        }
        if (!from_hole) {
            ensure_arena(used_ + n);
            used_ += n;
        }
        free_ranges_.erase(std::remove_if(free_ranges_.begin(), free_ranges_.end(),
                                          [](const std::pair<uint32_t, uint32_t>& h) { return h.second == 0; }),
                           free_ranges_.end());
        s.n = n;
        s.sbase = sbase;
        s.buckets = buckets_for(n);
        FLK_CUDA(cudaStreamWaitEvent(stream_, landed, 0));
        const int blocks = std::min<uint32_t>((n + 255) / 256, (uint32_t)num_sms_ * 8);
        k_unpack<<<blocks, 256, 0, stream_>>>(stage, n, sbase, ar_);  // buffer 0
        FLK_CUDA(cudaGetLastError());
        FLK_CUDA(cudaFreeAsync(stage, stream_));
        FLK_CUDA(cudaEventDestroy(landed));
    }
    return id;
}

void Engine::read_flock_async(int id, float* time, float* words, cudaEvent_t done) {
    if (!has_flock(id)) throw Error{-4, "unknown flock id"};
    FLK_CUDA(cudaSetDevice(device_));
    sync_times();
    const Slot& s = slots_[id];
    if (time) *time = s.time;
    if (s.n) {
        // pack on the compute stream (ordered after the steps that wrote the
        // state), copy out on the copy stream while the next chunk runs
        const size_t bytes = (size_t)s.n * WORDS * 4;
        float* stage = nullptr;
        FLK_CUDA(cudaMallocAsync((void**)&stage, bytes, stream_));
        const int blocks = std::min<uint32_t>((s.n + 255) / 256, (uint32_t)num_sms_ * 8);
        k_pack<<<blocks, 256, 0, stream_>>>(stage, s.n, (s.parity & 1u) * cap_ + s.sbase, ar_);
        FLK_CUDA(cudaGetLastError());
        cudaEvent_t packed;
        FLK_CUDA(cudaEventCreateWithFlags(&packed, cudaEventDisableTiming));
        FLK_CUDA(cudaEventRecord(packed, stream_));
        FLK_CUDA(cudaStreamWaitEvent(copy_, packed, 0));
        FLK_CUDA(cudaMemcpyAsync(words, stage, bytes, cudaMemcpyDeviceToHost, copy_));
        FLK_CUDA(cudaFreeAsync(stage, copy_));
        FLK_CUDA(cudaEventDestroy(packed));
    }
    FLK_CUDA(cudaEventRecord(done, copy_));
}

void Engine::read_flock(int id, float* time, float* words) {
    if (!has_flock(id)) throw Error{-4, "unknown flock id"};
    FLK_CUDA(cudaSetDevice(device_));
    sync_times();
    const Slot& s = slots_[id];
    if (time) *time = s.time;
    if (!s.n) return;
    const size_t bytes = (size_t)s.n * WORDS * 4;
    if (bytes > staging_cap_) {
        dev_bytes_ -= staging_cap_;
        dfree(staging_);
        staging_ = dalloc<float>((size_t)s.n * WORDS, &dev_bytes_);
        staging_cap_ = bytes;
    }
    const int blocks = std::min<uint32_t>((s.n + 255) / 256, (uint32_t)num_sms_ * 8);
    k_pack<<<blocks, 256, 0, stream_>>>(staging_, s.n, (s.parity & 1u) * cap_ + s.sbase, ar_);
    FLK_CUDA(cudaGetLastError());
    FLK_CUDA(cudaMemcpyAsync(words, staging_, bytes, cudaMemcpyDeviceToHost, stream_));
    FLK_CUDA(cudaStreamSynchronize(stream_));
}

void Engine::set_remaining(const std::vector<int>& ids, const std::vector<uint32_t>& steps) {
    sync_times();
    for (auto& s : slots_) s.remaining = 0;
    for (size_t k = 0; k < ids.size(); ++k) {
        if (!has_flock(ids[k])) throw Error{-4, "unknown flock id"};
        slots_[ids[k]].remaining = steps[k];
    }
    table_dirty_ = true;
}

void Engine::set_flock_remaining(int id, uint32_t steps) {
    if (!has_flock(id)) throw Error{-4, "unknown flock id"};
    // a flock that is not in the device table has no device-side countdown to
    // read back, so the host need not wait for work in flight
    if (std::find(table_ids_.begin(), table_ids_.end(), id) != table_ids_.end()) sync_times();
    slots_[id].remaining = steps;
    table_dirty_ = true;
}

uint32_t Engine::flock_remaining(int id) {
    if (!has_flock(id)) throw Error{-4, "unknown flock id"};
    sync_times();
    return slots_[id].remaining;
}

std::vector<uint32_t> Engine::remaining_of(const std::vector<int>& ids) {
    sync_times();
    std::vector<uint32_t> out;
    for (int id : ids) {
        if (!has_flock(id)) throw Error{-4, "unknown flock id"};
        out.push_back(slots_[id].remaining);
    }
    return out;
}

double Engine::time_run(uint32_t steps) {
    FLK_CUDA(cudaSetDevice(device_));
    prepare(false);
    cudaEvent_t e0, e1;
    FLK_CUDA(cudaEventCreate(&e0));
    FLK_CUDA(cudaEventCreate(&e1));
    // capture (if needed) before the timed region so the events bracket launches only
    if (!table_h_.empty() && steps >= (uint32_t)std::max(1, shape_.graph_chunk)) ensure_graph();
    FLK_CUDA(cudaEventRecord(e0, stream_));
    run(steps);
    FLK_CUDA(cudaEventRecord(e1, stream_));
    FLK_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    FLK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

__global__ void k_flush(uint4* __restrict__ buf, size_t n16, uint32_t salt) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
        buf[i] = make_uint4(salt, (uint32_t)i, salt, (uint32_t)i);
}

void Engine::time_steps_cold(uint32_t steps, size_t flush_bytes, float* ms_per_step) {
    FLK_CUDA(cudaSetDevice(device_));
    prepare(false);
    if (table_h_.empty() || steps == 0) return;
    uint4* flush = nullptr;
    const size_t n16 = flush_bytes / 16;
    size_t flush_acct = 0;
    if (n16) flush = dalloc<uint4>(n16, &flush_acct);
    // Each timed step is one launch of a single-step graph that runs the step as
    // a multi-step run does: its integrate also counts the next step's grid, so
    // the step has no hash pass of its own. Steps alternate between the two grid
    // buffers, hence one graph per buffer. The first step's grid is counted
    // before the timed region and one untimed step after it consumes the grid
    // the last timed step counted: every timed step counts every bird once, and
    // both grid buffers end clear.
    cudaGraphExec_t one[2] = {nullptr, nullptr};
    for (int b = 0; b < 2; ++b) {
        cudaGraph_t g;
        FLK_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        enqueue_step(false, nullptr, false, b, false, true);
        FLK_CUDA(cudaStreamEndCapture(stream_, &g));
        cudaError_t e = cudaGraphInstantiate(&one[b], g, 0);
        cudaGraphDestroy(g);
        FLK_CUDA(e);
    }
    std::vector<cudaEvent_t> ev(2 * (size_t)steps);
    for (auto& x : ev) FLK_CUDA(cudaEventCreate(&x));
    enqueue_hash(0);
    for (uint32_t s = 0; s < steps; ++s) {
        if (n16) k_flush<<<num_sms_ * 4, 256, 0, stream_>>>(flush, n16, s);
        FLK_CUDA(cudaEventRecord(ev[2 * s], stream_));
        FLK_CUDA(cudaGraphLaunch(one[s & 1u], stream_));
        FLK_CUDA(cudaEventRecord(ev[2 * s + 1], stream_));
    }
    enqueue_step(false, nullptr, false, (int)(steps & 1u), false, false);
    FLK_CUDA(cudaGetLastError());
    FLK_CUDA(cudaStreamSynchronize(stream_));
    for (uint32_t s = 0; s < steps; ++s) FLK_CUDA(cudaEventElapsedTime(&ms_per_step[s], ev[2 * s], ev[2 * s + 1]));
    for (auto& x : ev) cudaEventDestroy(x);
    for (auto& x : one) cudaGraphExecDestroy(x);
    dfree(flush);
    const uint32_t ran = steps + 1;
    for (size_t k = 0; k < table_h_.size(); ++k) {
        const uint32_t left = table_h_[k].remaining > ran ? table_h_[k].remaining - ran : 0;
        table_h_[k].remaining = left;
        if (table_ids_[k] >= 0) slots_[table_ids_[k]].remaining = left;
    }
    table_dirty_ = true;
}

// Bucket count of a production step (one that reports no keys; any count
// gives the same sets): the power of two at or above n, at least 2^12 (a
// lattice of at least 16 cells per axis) and at most 2^27. At the flock's
// density (0.5 birds per m^3, 32 birds per occupied cell) the lattice holds
// 32 times the flock's volume, so only a flock that spreads far wraps it.
uint32_t production_buckets(uint32_t n) {
    uint64_t want = 1;
    while (want < (uint64_t)n) want <<= 1;
    return (uint32_t)std::min<uint64_t>(std::max<uint64_t>(want, 1u << 12), 1u << 27);
}

void Engine::prepare(bool grid_output) {
    if (table_dirty_ || table_grid_output_ != grid_output) {
        sync_times();
        rebuild_table(grid_output);
    }
}

void Engine::rebuild_table(bool grid_output) {
    table_grid_output_ = grid_output;
    std::vector<FlockDesc> t;
    std::vector<int> ids;
    uint32_t V = 0;
    uint64_t Bt = 0;
    for (size_t k = 0; k < slots_.size(); ++k) {
        const Slot& s = slots_[k];
        if (!s.live || s.remaining == 0) continue;
        FlockDesc d{};
        d.vbase = V;
        d.n = s.n;
        d.sbase = s.sbase;
        d.bbase = (uint32_t)Bt;
        d.buckets = grid_output ? s.buckets : production_buckets(s.n);
        d.remaining = s.remaining;
        d.time = s.time;
        d.parity = s.parity;
        t.push_back(d);
        ids.push_back((int)k);
        V += s.n;
        Bt += d.buckets;
    }
    if (Bt >= (1ull << 32) - SCAN_TILE) throw Error{-5, "too many buckets in one batch"};
    if ((uint32_t)t.size() > table_cap_ || !table_d_) {
        dev_bytes_ -= (size_t)table_cap_ * sizeof(FlockDesc);
        dfree(table_d_);
        table_cap_ = std::max<uint32_t>((uint32_t)t.size(), 16);
        table_d_ = dalloc<FlockDesc>(table_cap_, &dev_bytes_);
    }
    if (!t.empty())
        FLK_CUDA(cudaMemcpyAsync(table_d_, t.data(), t.size() * sizeof(FlockDesc), cudaMemcpyHostToDevice, stream_));
    // a captured graph bakes in sizes and pointers, not the table contents
    const bool same_shape = t.size() == table_h_.size() && V == V_ && (uint32_t)Bt == Btot_;
    table_h_ = t;
    table_ids_ = ids;
    V_ = V;
    Btot_ = (uint32_t)Bt;
    if (!same_shape) free_graphs();
    ensure_scratch();
    table_dirty_ = false;
    device_ahead_ = false;  // the device table now equals the host copy
}

void Engine::ensure_scratch() {
    if (V_ > scratch_V_ || !key_) {
        const uint32_t nv = std::max<uint32_t>(V_, scratch_V_ + scratch_V_ / 2);
        dev_bytes_ -= (size_t)scratch_V_ * 88;
        if (sets_) dev_bytes_ -= (size_t)scratch_V_ * 32;
        dfree(key_); dfree(arrival_); dfree(tmp_); dfree(occ_); dfree(occ2_); dfree(due_);
        dfree(sfwd_); dfree(sets_);
        key_ = dalloc<uint32_t>(nv, &dev_bytes_);
        arrival_ = dalloc<uint32_t>(nv, &dev_bytes_);
        tmp_ = dalloc<unsigned long long>(nv, &dev_bytes_);
        occ_ = dalloc<uint32_t>(nv, &dev_bytes_);
        occ2_ = dalloc<uint32_t>(nv, &dev_bytes_);
        due_ = dalloc<DueRec>(nv, &dev_bytes_);
        sfwd_ = dalloc<float4>(nv, &dev_bytes_);
        scratch_V_ = nv;
        free_graphs();
    }
    if (Btot_ > scratch_B_) {
        const uint32_t nb = Btot_;
        dev_bytes_ -= (size_t)scratch_B_ * 16 + (scratch_B_ / SCAN_TILE) * 8;
        dfree(counts_); dfree(counts2_); dfree(offsets_); dfree(status_); dfree(slabs_);
        counts_ = dalloc<uint32_t>(nb, &dev_bytes_);
        counts2_ = dalloc<uint32_t>(nb, &dev_bytes_);
        slabs_ = dalloc<uint32_t>(nb, &dev_bytes_);
        offsets_ = dalloc<uint32_t>((size_t)nb + 1, &dev_bytes_);
        status_ = dalloc<unsigned long long>(nb / SCAN_TILE, &dev_bytes_);
        FLK_CUDA(cudaMemsetAsync(counts_, 0, (size_t)nb * 4, stream_));
        FLK_CUDA(cudaMemsetAsync(counts2_, 0, (size_t)nb * 4, stream_));
        FLK_CUDA(cudaMemsetAsync(status_, 0, (size_t)(nb / SCAN_TILE) * 8, stream_));
        scratch_B_ = nb;
        free_graphs();
    }
}

// Grid of a persistent pass: `per_sm` CTAs per SM, but no more CTAs than
// there are work items (`items` split into `per_cta` per CTA).
static int pgrid(int sms, int per_sm, uint64_t items, uint64_t per_cta) {
    const uint64_t need = (items + per_cta - 1) / per_cta;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * per_sm, need));
}

GridBuf Engine::grid_buf(int k) const {
    return k ? GridBuf{counts2_, occ2_, &ctl_->occ_count[1]} : GridBuf{counts_, occ_, &ctl_->occ_count[0]};
}

void Engine::enqueue_step(bool sets, cudaEvent_t* ev, bool f64, int buf, bool hash, bool fuse_next) {
    device_ahead_ = true;
    const int nfl = (int)table_h_.size();
    // grid of a bird-parallel pass whose kernel fits `f` CTAs per SM
    auto sgrid = [&](int f) { return pgrid(num_sms_, std::min(shape_.stream_blocks_per_sm, f), V_, 256); };
    const uint32_t ntiles = Btot_ / SCAN_TILE;
    const GridBuf g = grid_buf(buf), gn = grid_buf(buf ^ 1);
    const float cell = shape_.cell, inv_cell = 1.0f / shape_.cell;  // production cells
    if (ev) FLK_CUDA(cudaEventRecord(ev[0], stream_));
    if (sets)  // a grid-reporting step: the reference's cell hash
        k_hash_count<false><<<sgrid(fit_.hash[0]), 256, 0, stream_>>>(table_d_, nfl, V_, ar_, key_, arrival_, g, ctl_,
                                                                      INV_CELL);
    else if (hash)
        enqueue_hash(buf);
    if (ev) FLK_CUDA(cudaEventRecord(ev[1], stream_));
    if (sets) {
        // a step that reports its grid builds the canonical dense offsets
        // (every bucket, in bucket order) and uses them as the run starts
        k_scan<<<ntiles, SCAN_THREADS, 0, stream_>>>(g.counts, offsets_, ntiles, status_, ctl_);
    } else {
        k_place<<<pgrid(num_sms_, std::min(shape_.stream_blocks_per_sm, fit_.place), Btot_, 1024), 256, 0, stream_>>>(
            table_d_, nfl, Btot_, g.counts, offsets_, g.occ, g.occ_count);
    }
    if (ev) FLK_CUDA(cudaEventRecord(ev[2], stream_));
    k_scatter<<<sgrid(fit_.scatter), 256, 0, stream_>>>(table_d_, nfl, V_, ar_, key_, arrival_, offsets_, tmp_, ctl_);
    k_segsort<<<pgrid(num_sms_, std::min(shape_.segsort_blocks_per_sm, fit_.segsort), V_, 8), 256, 0, stream_>>>(
        table_d_, nfl, V_, ctl_, g.occ, offsets_, g.counts, g.occ_count, tmp_, ar_, sfwd_, due_, slabs_);
    if (f64) {  // FP64 evaluation from the input state, before the f32 passes change it
        k_decide_f64<<<pgrid(num_sms_, fit_.decide_f64, V_, 8), 256, 0, stream_>>>(table_d_, nfl, V_, ctl_, due_, offsets_,
                                                                      g.counts, ar_, dec64_, err64_, cell, inv_cell);
        k_integrate_f64<<<sgrid(fit_.integrate_f64), 256, 0, stream_>>>(table_d_, nfl, V_, ar_, dec64_, out64_);
    }
    if (ev) FLK_CUDA(cudaEventRecord(ev[3], stream_));
    const int dblocks = pgrid(num_sms_, shape_.decide_blocks_per_sm, V_, shape_.decide_threads / 32);
    // per-warp hit queue + reduced birds awaiting their epilogue (+ any reserved extra)
    const size_t qbytes = decide_smem(sets);
    if (sets)
        k_decide<true><<<dblocks, shape_.decide_threads, qbytes, stream_>>>(table_d_, nfl, V_, ctl_, due_, offsets_,
                                                                       g.counts, ar_, sfwd_, radius_table_, sets_,
                                                                       slabs_, GRID_CELL, INV_CELL);
    else if (shape_.decide_kind == 1)
        k_decide_staged<<<dblocks, shape_.decide_threads, qbytes, stream_>>>(table_d_, nfl, V_, ctl_, due_, offsets_,
                                                                            g.counts, ar_, sfwd_, radius_table_,
                                                                            slabs_, cell, inv_cell, STAGE_CAP);
    else
        k_decide<false><<<dblocks, shape_.decide_threads, qbytes, stream_>>>(table_d_, nfl, V_, ctl_, due_, offsets_,
                                                                        g.counts, ar_, sfwd_, radius_table_, nullptr,
                                                                        slabs_, cell, inv_cell);
    if (ev) FLK_CUDA(cudaEventRecord(ev[4], stream_));
    if (fuse_next && !sets)
        k_integrate<true><<<sgrid(fit_.integrate[1]), 256, 0, stream_>>>(table_d_, nfl, V_, ar_, g, gn, key_, arrival_, ctl_,
                                                                         inv_cell);
    else
        k_integrate<false><<<sgrid(fit_.integrate[0]), 256, 0, stream_>>>(table_d_, nfl, V_, ar_, g, gn, key_, arrival_, ctl_,
                                                                          inv_cell);
    if (f64) k_compare_f64<<<sgrid(fit_.compare_f64), 256, 0, stream_>>>(table_d_, nfl, V_, ar_, active_, out64_, err64_);
    if (ev) FLK_CUDA(cudaEventRecord(ev[5], stream_));
}

void Engine::enqueue_hash(int buf) {
    device_ahead_ = true;
    const int grid = pgrid(num_sms_, std::min(shape_.stream_blocks_per_sm, fit_.hash[1]), V_, 256);
    k_hash_count<true><<<grid, 256, 0, stream_>>>(table_d_, (int)table_h_.size(), V_, ar_, key_, arrival_,
                                                  grid_buf(buf), ctl_, 1.0f / shape_.cell);
}

void Engine::enqueue_steps(uint32_t n) {
    for (uint32_t i = 0; i < n; ++i) enqueue_step(false, nullptr, false, (int)(i & 1u), i == 0, i + 1 < n);
}

// A chunk of `graph_chunk` steps as one CUDA graph. When only sizes, pointers
// or launch shapes changed since the last capture (a flock joined or left, a
// buffer grew), the new capture has the same nodes, and cudaGraphExecUpdate
// rewrites the executable graph's parameters instead of instantiating a new
// one (launches already in flight keep their old parameters). A different
// chunk length, or an update the runtime refuses, instantiates afresh.
void Engine::ensure_graph() {
    const uint32_t chunk = (uint32_t)std::max(1, shape_.graph_chunk);
    if (graph_ && graph_steps_ == chunk && !graph_stale_) return;
    cudaGraph_t g;
    FLK_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    enqueue_steps(chunk);
    FLK_CUDA(cudaStreamEndCapture(stream_, &g));
    if (graph_ && graph_steps_ == chunk) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(graph_, g, &info) == cudaSuccess) {
            cudaGraphDestroy(g);
            graph_stale_ = false;
            ++graph_updates_;
            return;
        }
        (void)cudaGetLastError();  // the refused update leaves no sticky error
    }
    destroy_graphs();
    cudaError_t e = cudaGraphInstantiate(&graph_, g, 0);
    cudaGraphDestroy(g);
    FLK_CUDA(e);
    graph_steps_ = chunk;
    ++graph_instantiations_;
}

void Engine::run(uint32_t steps) {
    FLK_CUDA(cudaSetDevice(device_));
    prepare(false);
    if (table_h_.empty() || steps == 0) return;
    const uint32_t chunk = (uint32_t)std::max(1, shape_.graph_chunk);
    uint32_t done = 0;
    if (steps >= chunk) {
        // A chunk graph that must be captured (first run, or the flock table
        // changed) costs host time. With at least two chunks to run, the first
        // chunk goes out as plain launches and the capture runs on the host
        // while the GPU executes them; the launches are the captured ones, so
        // the results are the same.
        if (steps >= 2 * chunk && (!graph_ || graph_steps_ != chunk || graph_stale_)) {
            enqueue_steps(chunk);
            done = chunk;
        }
        ensure_graph();
        device_ahead_ = true;
        for (; done + chunk <= steps; done += chunk) FLK_CUDA(cudaGraphLaunch(graph_, stream_));
    }
    if (done < steps) enqueue_steps(steps - done);
    FLK_CUDA(cudaGetLastError());
    // host mirror of the countdown (clocks are read back on demand)
    bool finished = false;
    for (size_t k = 0; k < table_h_.size(); ++k) {
        const uint32_t left = table_h_[k].remaining > steps ? table_h_[k].remaining - steps : 0;
        table_h_[k].remaining = left;
        if (table_ids_[k] >= 0) slots_[table_ids_[k]].remaining = left;
        finished |= left == 0;
    }
    // flocks that reached zero leave the table at the next run (their clocks
    // are read back from the device table before it is rebuilt)
    if (finished) table_dirty_ = true;
}

void Engine::run_timed(uint32_t steps, uint32_t warmup, PassTimes* out) {
    FLK_CUDA(cudaSetDevice(device_));
    prepare(false);
    PassTimes pt{};
    if (table_h_.empty() || steps == 0) {
        if (out) *out = pt;
        return;
    }
    std::vector<cudaEvent_t> ev((size_t)steps * 6);
    for (auto& e : ev) FLK_CUDA(cudaEventCreate(&e));
    for (uint32_t s = 0; s < steps; ++s) enqueue_step(false, &ev[(size_t)s * 6]);
    FLK_CUDA(cudaGetLastError());
    FLK_CUDA(cudaStreamSynchronize(stream_));
    warmup = std::min(warmup, steps);
    for (uint32_t s = warmup; s < steps; ++s) {
        cudaEvent_t* e = &ev[(size_t)s * 6];
        for (int p = 0; p < 5; ++p) {
            float ms = 0;
            FLK_CUDA(cudaEventElapsedTime(&ms, e[p], e[p + 1]));
            pt.ms[p] += ms;
        }
    }
    pt.timed_steps = (int)(steps - warmup);
    if (pt.timed_steps > 0) {
        for (int p = 0; p < 5; ++p) {
            pt.ms[p] /= pt.timed_steps;
            pt.total_ms += pt.ms[p];
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    sync_times();  // clocks and countdowns from the device table
    table_dirty_ = true;
    if (out) *out = pt;
}

void Engine::step_debug(std::vector<GridDebug>* out) {
    FLK_CUDA(cudaSetDevice(device_));
    prepare(true);  // the canonical bucket counts the reported grid is defined with
    if (table_h_.empty()) return;
    if (!sets_) sets_ = dalloc<uint32_t>((size_t)scratch_V_ * 8, &dev_bytes_);
    FLK_CUDA(cudaMemsetAsync(sets_, 0, (size_t)V_ * 8 * 4, stream_));
    const std::vector<FlockDesc> before = table_h_;
    enqueue_step(true);
    FLK_CUDA(cudaGetLastError());
    FLK_CUDA(cudaStreamSynchronize(stream_));
    // a grid the device gave up on is not interpreted
    if (const uint32_t err = check_device_error()) {
        table_dirty_ = true;
        device_ahead_ = true;
        throw Error{-6, std::string("device: ") + device_error_text(err)};
    }
    std::vector<uint32_t> key(V_), offs((size_t)Btot_ + 1), sets((size_t)V_ * 8);
    FLK_CUDA(cudaMemcpy(key.data(), key_, (size_t)V_ * 4, cudaMemcpyDeviceToHost));
    FLK_CUDA(cudaMemcpy(offs.data(), offsets_, ((size_t)Btot_ + 1) * 4, cudaMemcpyDeviceToHost));
    FLK_CUDA(cudaMemcpy(sets.data(), sets_, (size_t)V_ * 8 * 4, cudaMemcpyDeviceToHost));
    // bird index per slot in both buffers: the step read buf[parity] (keys are
    // per old slot) and wrote buf[parity ^ 1] (sorted order, sets per new slot)
    std::vector<uint32_t> ids[2];
    for (int k = 0; k < 2; ++k) {
        ids[k].resize(used_);
        if (used_)
            FLK_CUDA(cudaMemcpy(ids[k].data(), ar_.id + (size_t)k * cap_, (size_t)used_ * 4, cudaMemcpyDeviceToHost));
    }
    out->clear();
    for (const FlockDesc& d : before) {
        const std::vector<uint32_t>& oid = ids[d.parity & 1u];
        const std::vector<uint32_t>& nid = ids[(d.parity & 1u) ^ 1u];
        GridDebug g;
        g.keys.assign(d.n, 0);
        g.sets.assign((size_t)d.n * 8, 0);
        g.sorted.resize(d.n);
        for (uint32_t i = 0; i < d.n; ++i) {
            const uint32_t bo = oid[d.sbase + i], bn = nid[d.sbase + i];
            if (bo >= d.n || bn >= d.n) throw Error{-6, "bird index out of range in step_debug"};
            g.keys[bo] = key[d.vbase + i] - d.bbase;
            g.sorted[i] = bn;  // view index vbase + i holds bird bn
            std::copy(sets.begin() + (size_t)(d.vbase + i) * 8, sets.begin() + (size_t)(d.vbase + i + 1) * 8,
                      g.sets.begin() + (size_t)bn * 8);
        }
        g.offsets.resize((size_t)d.buckets + 1);
        const uint32_t o0 = offs[d.bbase];
        for (uint32_t b = 0; b <= d.buckets; ++b) g.offsets[b] = offs[(size_t)d.bbase + b] - o0;
        if (o0 != d.vbase) throw Error{-6, "grid offsets of a flock do not start at its view base"};
        out->push_back(std::move(g));
    }
    sync_times();  // clocks and countdowns from the device table
    table_dirty_ = true;
}

void Engine::step_f64(std::vector<std::vector<double>>* out, std::vector<std::array<double, 4>>* report) {
    FLK_CUDA(cudaSetDevice(device_));
    prepare(false);  // production buckets: the FP64 passes use the lattice index
    out->clear();
    report->clear();
    if (table_h_.empty()) return;
    if (V_ > f64_V_ || !dec64_) {
        dfree(dec64_);
        dfree(out64_);
        dec64_ = dalloc<double>((size_t)V_ * 8, &dev_bytes_);
        out64_ = dalloc<double>((size_t)V_ * 15, &dev_bytes_);
        f64_V_ = V_;
    }
    const size_t nfl = table_h_.size();
    if (nfl > active_cap_ || !active_) {
        dfree(active_);
        dfree(err64_);
        active_cap_ = (uint32_t)nfl;
        active_ = dalloc<uint8_t>(active_cap_, &dev_bytes_);
        err64_ = dalloc<uint32_t>((size_t)active_cap_ * 4, &dev_bytes_);
    }
    const std::vector<FlockDesc> before = table_h_;
    std::vector<uint8_t> act(nfl);
    for (size_t k = 0; k < nfl; ++k) act[k] = before[k].remaining > 0;
    FLK_CUDA(cudaMemcpyAsync(active_, act.data(), nfl, cudaMemcpyHostToDevice, stream_));
    FLK_CUDA(cudaMemsetAsync(err64_, 0, nfl * 16, stream_));
    enqueue_step(false, nullptr, true);
    FLK_CUDA(cudaGetLastError());
    std::vector<uint32_t> err(nfl * 4);
    FLK_CUDA(cudaMemcpyAsync(err.data(), err64_, nfl * 16, cudaMemcpyDeviceToHost, stream_));
    std::vector<double> o64((size_t)V_ * 15);
    FLK_CUDA(cudaMemcpyAsync(o64.data(), out64_, o64.size() * 8, cudaMemcpyDeviceToHost, stream_));
    std::vector<uint32_t> ids[2];
    for (int k = 0; k < 2; ++k) {
        ids[k].resize(used_);
        if (used_)
            FLK_CUDA(cudaMemcpyAsync(ids[k].data(), ar_.id + (size_t)k * cap_, (size_t)used_ * 4,
                                     cudaMemcpyDeviceToHost, stream_));
    }
    FLK_CUDA(cudaStreamSynchronize(stream_));
    for (size_t f = 0; f < nfl; ++f) {
        const FlockDesc& d = before[f];
        std::vector<double> w;
        std::array<double, 4> r{0.0, 0.0, 0.0, 0.0};
        if (d.remaining) {
            float ep, ev;
            std::memcpy(&ep, &err[4 * f], 4);
            std::memcpy(&ev, &err[4 * f + 1], 4);
            r = {ep, ev, (double)err[4 * f + 2], (double)err[4 * f + 3]};
            // view index vbase + i sits in slot sbase + i of the copy the step wrote
            const std::vector<uint32_t>& nid = ids[(d.parity & 1u) ^ 1u];
            w.resize((size_t)d.n * 15);
            for (uint32_t i = 0; i < d.n; ++i) {
                const uint32_t bird = nid[d.sbase + i];
                if (bird >= d.n) throw Error{-6, "bird index out of range in step_f64"};
                std::memcpy(&w[(size_t)bird * 15], &o64[(size_t)(d.vbase + i) * 15], 15 * 8);
            }
        }
        out->push_back(std::move(w));
        report->push_back(r);
    }
}

void Engine::sync() {
    FLK_CUDA(cudaSetDevice(device_));
    FLK_CUDA(cudaStreamSynchronize(stream_));
}

uint32_t Engine::check_device_error() {
    FLK_CUDA(cudaSetDevice(device_));
    StepCtl c;
    FLK_CUDA(cudaMemcpyAsync(&c, ctl_, sizeof c, cudaMemcpyDeviceToHost, stream_));
    FLK_CUDA(cudaStreamSynchronize(stream_));
    if (c.error) {
        const uint32_t z = 0;
        FLK_CUDA(cudaMemcpyAsync(&ctl_->error, &z, 4, cudaMemcpyHostToDevice, stream_));
        FLK_CUDA(cudaStreamSynchronize(stream_));
    }
    return c.error;
}

void Engine::arm_scan_timeout(uint32_t skip_tile, uint32_t spin_limit) {
    FLK_CUDA(cudaSetDevice(device_));
    const uint32_t v[2] = {skip_tile + 1u, spin_limit};
    FLK_CUDA(cudaMemcpyAsync(&ctl_->scan_skip1, v, sizeof v, cudaMemcpyHostToDevice, stream_));
    FLK_CUDA(cudaStreamSynchronize(stream_));
}

void Engine::counters(unsigned long long* due, unsigned long long* cand, unsigned long long* pairs) {
    FLK_CUDA(cudaSetDevice(device_));
    StepCtl c;
    FLK_CUDA(cudaMemcpyAsync(&c, ctl_, sizeof c, cudaMemcpyDeviceToHost, stream_));
    FLK_CUDA(cudaStreamSynchronize(stream_));
    if (due) *due = c.due_total;
    if (cand) *cand = c.cand_total;
    if (pairs) *pairs = c.pair_total;
}

}  // namespace flk

