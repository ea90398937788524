// Internal C++ interface of the GB300 flock engine: a resident arena of one
// or more flocks and the per-step passes that advance all of them in one
// launch per pass. The plain single-flock step, the batched step and the
// serving pool are all this engine with one, many or a changing set of flocks,
// so a flock's result does not depend on what else is resident.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <array>
#include <string>
#include <vector>

namespace flk {

// One flock in the device flock table (rebuilt whenever the resident set changes).
struct FlockDesc {
    uint32_t vbase;      // first virtual bird index (concatenation of table entries)
    uint32_t n;          // birds
    uint32_t sbase;      // first storage slot in the arena
    uint32_t bbase;      // first global bucket
    uint32_t buckets;    // power of two, buckets_for(n)
    uint32_t remaining;  // steps still to run; 0 = idle this step
    float time;          // world clock (f32, as the reference keeps it)
    uint32_t cursor;     // next free slot of the flock's view region (bucket allocation; reset per step)
    uint32_t parity;     // which of the two state buffers holds the flock's current state
    uint32_t pad[3];
};

// The arena's state, two copies: buffer p of each field occupies entries
// [p * cap, (p + 1) * cap). A = position, roll; B = velocity, spin; C =
// steering, radius; D = next_decision, neighbours (u32 bits), centrality;
// id = the bird's index in its flock. Each step reads a flock's state from
// buffer `parity` and writes it, reordered by cell, into buffer parity ^ 1, so
// consecutive slots hold birds of the same cell (coherent gathers,
// warp-aggregated atomics, and the candidate view for decide is the state
// itself). Slot of view index v of a flock in buffer p: v + p * cap + sbase - vbase.
struct Arena {
    float4* A;
    float4* B;
    float4* C;
    float4* D;
    uint32_t* id;
    uint32_t cap;
};

// Step-control block in device memory: per-step counters (reset by the last
// block of the integrate pass), the scan epoch and the device error word.
struct StepCtl {
    uint32_t occ_count[2];  // occupied buckets found, per grid buffer
    uint32_t due_count;    // deciding birds this step
    uint32_t scan_ticket;  // dynamic tile ids of the scan
    uint32_t epoch;        // scan status tag, advanced once per step
    uint32_t done_blocks;  // integrate's last-block detector
    uint32_t error;        // first device error (FLK_DEV_*), 0 = none
    uint32_t err_info;
    unsigned long long due_total;   // cumulative deciding birds
    unsigned long long cand_total;  // cumulative candidate tests in decide
    unsigned long long pair_total;  // cumulative pairs inside 2R
    // Test hook, one step only (the next grid-reporting step's scan; integrate's
    // last block clears both): scan tile scan_skip1 - 1 publishes no status
    // flag (0 = none), so the tiles after it wait for a flag nothing sets;
    // scan_spin, if non-zero, replaces the look-back's poll limit.
    uint32_t scan_skip1;
    uint32_t scan_spin;
};

// One of the two grid buffers: the histogram (run lengths, per bucket), the
// occupied-bucket list and its length. A multi-step run alternates them so
// that a step's integrate can count the next step's grid while its own is
// cleared.
struct GridBuf {
    uint32_t* counts;
    uint32_t* occ;
    uint32_t* occ_count;
};

// One deciding bird, written by the per-bucket sort so that decide can start
// from a single record (48 B, three 16-byte loads from one place).
struct __align__(16) DueRec {
    float4 pr;  // position xyz, radius
    float4 fk;  // unit heading xyz, index in the cell-ordered view (u32 bits)
    uint4 fl;   // slot in the reordered buffer, bucket base, bucket count, slot - view index of that buffer
};

enum DeviceError : uint32_t {
    DEV_OK = 0,
    DEV_SCAN_TIMEOUT = 1,  // a scan look-back wait gave up
    DEV_BAD_RANGE = 2,     // a bucket range or slot fell outside its array (skipped, not accessed)
    DEV_STAGE_TIMEOUT = 3, // a staged decide's bulk copies did not land within the wait limit
};

// Per-pass timing of a step, mean ms over the timed steps (reference's table).
struct PassTimes {
    double ms[5];  // hash+count, scan, scatter+segment sort, decide, integrate
    double total_ms;
    int timed_steps;
};

// Sizes of the engine's launch shapes; chosen by the autotuner or defaults.
struct LaunchShape {
    int stream_blocks_per_sm = 8;   // bird-parallel passes: 256-thread CTAs per SM
    int decide_threads = 1024;      // threads per decide CTA
    int decide_blocks_per_sm = 1;   // decide CTAs per SM
    int segsort_blocks_per_sm = 8;  // segment-sort CTAs per SM (256 threads)
    int graph_chunk = 10;           // steps per captured CUDA graph
    size_t decide_extra_smem = 0;   // dynamic shared memory reserved beyond decide's own (occupancy experiments)
    float cell = 4.0f;              // production cell edge (m); any edge gives the same neighbour sets
    int decide_kind = 0;            // production decide: 0 sweeps the state, 1 stages cells in shared memory
};

struct GridDebug {  // host copies of one step's grid and neighbour-set summaries
    std::vector<uint32_t> keys, offsets, sorted;  // per flock: n, buckets+1, n
    std::vector<uint32_t> sets;                   // 8 words per bird (zeros for non-deciding birds)
};

class Engine {
public:
    explicit Engine(int device = -1);
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    // Flocks. `words` is a host array of n*15 .flk words (any host memory).
    int add_flock(uint32_t n, float time, const float* words);  // returns id >= 0
    // Same, but the host-to-device copy runs on the copy stream and overlaps
    // the compute stream's work; `words` must stay valid until the next sync.
    int add_flock_async(uint32_t n, float time, const float* words);
    // Packs the flock on the compute stream and copies it out on the copy
    // stream; `done` (an event) is recorded when `words` holds the result.
    // The slot may be removed right after the call (stream order protects it).
    void read_flock_async(int id, float* time, float* words, cudaEvent_t done);
    void remove_flock(int id);
    void read_flock(int id, float* time, float* words);  // D2H + pack
    float flock_time(int id);
    uint32_t flock_size(int id) const;
    bool has_flock(int id) const;
    std::vector<int> flock_ids() const;

    // Sets how many steps each listed flock still has to run (others: 0).
    void set_remaining(const std::vector<int>& ids, const std::vector<uint32_t>& steps);
    // Sets one flock's remaining steps, leaving the others as they are.
    void set_flock_remaining(int id, uint32_t steps);
    uint32_t flock_remaining(int id);
    std::vector<uint32_t> remaining_of(const std::vector<int>& ids);  // one device read for all
    // run(steps) bracketed by CUDA events on the engine stream; returns ms.
    double time_run(uint32_t steps);
    // `steps` single-step graph launches, each after overwriting `flush_bytes`
    // of device memory (cold L2), each bracketed by events; ms per step. Each
    // step runs as in a multi-step run (its integrate counts the next step's
    // grid); one untimed step follows, so the flock advances steps + 1 and
    // needs that many remaining.
    void time_steps_cold(uint32_t steps, size_t flush_bytes, float* ms_per_step);
    // Runs `steps` batched steps over the resident flocks (each flock stops
    // when its remaining count reaches zero). Uses captured CUDA graphs.
    void run(uint32_t steps);
    // Eager steps with per-pass events (the reference's timing table).
    void run_timed(uint32_t steps, uint32_t warmup, PassTimes* out);
    // One eager step that also returns every flock's grid and set summaries.
    void step_debug(std::vector<GridDebug>* out);
    // One production step of every active flock that also evaluates the same
    // step in FP64 from the same input state. Per table flock k (empty for
    // flocks that did not step): out[k] (bird order, n*15) receives the FP64
    // post-step state, report[k] = {max relative position error, max
    // relative velocity error, neighbour-count mismatches, deciding birds}
    // of its f32 step against it.
    void step_f64(std::vector<std::vector<double>>* out, std::vector<std::array<double, 4>>* report);
    void sync();
    uint32_t check_device_error();  // returns and clears the device error word
    // Test hook for the bounded device waits: in the next grid-reporting step,
    // scan tile `skip_tile` publishes no look-back flag and every look-back
    // gives up after `spin_limit` polls (0: the usual limit). The step then
    // ends with the device error word set to DEV_SCAN_TIMEOUT.
    void arm_scan_timeout(uint32_t skip_tile, uint32_t spin_limit);

    cudaStream_t stream() const { return stream_; }
    int device() const { return device_; }
    int num_sms() const { return num_sms_; }
    LaunchShape& shape() { return shape_; }
    void set_shape(const LaunchShape& s);
    // decide's launch as configured: resident CTAs per SM, threads per CTA and
    // dynamic shared memory per CTA (bytes), for production steps
    void decide_occupancy(int* blocks_per_sm, int* threads, size_t* smem_bytes) const;
    // decide's dynamic shared memory per CTA for a step kind (its own + the reserved extra)
    size_t decide_smem(bool sets) const;
    size_t device_bytes() const { return dev_bytes_; }
    // Cumulative counters from the step-control block.
    void counters(unsigned long long* due, unsigned long long* cand, unsigned long long* pairs);
    // Chunk graphs instantiated, and updated in place, so far.
    void graph_counts(uint64_t* instantiated, uint64_t* updated) const {
        *instantiated = graph_instantiations_;
        *updated = graph_updates_;
    }
    // Bytes of device memory a flock of n birds would add (state + scratch).
    static size_t bytes_for(uint32_t n);
    // Launches of engine kernels per step (for the bench's launch count).
    static int kernels_per_step() { return 6; }

private:
    // device memory through the process-wide per-device cache
    template <class T>
    T* dalloc(size_t n, size_t* acct);
    template <class T>
    void dfree(T*& p);
    struct Slot {
        uint32_t n = 0, sbase = 0, buckets = 0, remaining = 0;
        uint32_t parity = 0;  // buffer holding the current state
        float time = 0.f;
        bool live = false;
    };
    void ensure_arena(uint32_t need);
    void rebuild_table(bool grid_output);
    void prepare(bool grid_output);  // rebuild the table if stale or built for the other mode
    void ensure_scratch();
    // One step. `buf`: the grid buffer it uses; `hash`: count its grid here
    // (otherwise the previous step's integrate did); `fuse_next`: its integrate
    // also counts the next step's grid into the other buffer.
    void enqueue_step(bool sets, cudaEvent_t* ev = nullptr, bool f64 = false, int buf = 0, bool hash = true,
                      bool fuse_next = false);
    // `n` production steps, each integrate counting the next step's grid (the
    // first step counts its own, the last one counts none).
    void enqueue_steps(uint32_t n);
    // The production hash and count of the current positions into grid buffer `buf`.
    void enqueue_hash(int buf);
    GridBuf grid_buf(int k) const;
    void free_graphs();
    void destroy_graphs();
    void ensure_graph();
    void sync_times();

    int device_ = 0, num_sms_ = 0;
    cudaStream_t stream_ = nullptr;
    cudaStream_t copy_ = nullptr;  // host<->device state copies of the serving pool
    LaunchShape shape_;
    // 256-thread CTAs of each grid-stride kernel that fit on one SM at once
    // (occupancy API, from registers and shared memory); grids never exceed
    // them, so no CTA waits for a second wave
    struct Fit {
        int hash[2] = {8, 8}, place = 8, scatter = 8, segsort = 8, integrate[2] = {8, 8};
        int decide_f64 = 8, integrate_f64 = 8, compare_f64 = 8;
    } fit_;
    size_t dev_bytes_ = 0;

    // arena (storage order)
    uint32_t cap_ = 0, used_ = 0;
    Arena ar_{};  // two state buffers, cap_ birds each
    std::vector<Slot> slots_;
    std::vector<std::pair<uint32_t, uint32_t>> free_ranges_;  // (sbase, n) holes

    // flock table of flocks with remaining > 0, in slot order
    bool table_dirty_ = true;
    bool table_grid_output_ = false;  // table built with canonical bucket counts (grid-reporting step)
    bool device_ahead_ = false;  // steps ran since the host last read the device table
    std::vector<FlockDesc> table_h_;
    std::vector<int> table_ids_;
    FlockDesc* table_d_ = nullptr;
    uint32_t table_cap_ = 0;
    uint32_t V_ = 0, Btot_ = 0;

    // scratch (virtual / sorted order)
    uint32_t scratch_V_ = 0, scratch_B_ = 0;
    uint32_t *key_ = nullptr, *arrival_ = nullptr, *occ_ = nullptr;
    unsigned long long* tmp_ = nullptr;  // sort keys: bird << 32 | view index
    DueRec* due_ = nullptr;
    float4* sfwd_ = nullptr;  // unit heading per view index (read by decide)
    uint32_t *counts_ = nullptr, *offsets_ = nullptr;
    uint32_t *counts2_ = nullptr, *occ2_ = nullptr;  // the second grid buffer
    uint32_t* slabs_ = nullptr;  // per bucket: the run's z-slab boundaries (production steps)
    unsigned long long* status_ = nullptr;
    uint32_t* sets_ = nullptr;  // 8 per virtual bird, debug only
    StepCtl* ctl_ = nullptr;
    float* radius_table_ = nullptr;
    float* staging_ = nullptr;
    size_t staging_cap_ = 0;
    // FP64 evaluation (allocated on first use): decisions, post-step state,
    // per-flock active flags, error words
    double *dec64_ = nullptr, *out64_ = nullptr;
    uint32_t f64_V_ = 0;
    uint8_t* active_ = nullptr;
    uint32_t active_cap_ = 0;
    uint32_t* err64_ = nullptr;  // 4 words per table flock

    cudaGraphExec_t graph_ = nullptr;
    uint32_t graph_steps_ = 0;
    bool graph_stale_ = false;  // parameters changed since the capture (free_graphs)
    uint64_t graph_instantiations_ = 0, graph_updates_ = 0;
};

// Canonical bucket count for a flock of n birds (reference cuda/flock.cu:368-372).
uint32_t buckets_for(uint32_t n);
// Bucket count of a production step (the same rule without the 2^22 clamp).
uint32_t production_buckets(uint32_t n);

// What a device error word (DeviceError) means, as FLK_ERR_DEVICE reports it.
const char* device_error_text(uint32_t word);

// Device-error and CUDA failures surface as this exception inside the library;
// the C ABI turns it into a status code and a message.
struct Error {
    int code;
    std::string msg;
};

}  // namespace flk
