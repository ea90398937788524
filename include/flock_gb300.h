/*
 * flock_gb300.h -- C ABI of the GB300-native starling-flock step.
 *
 * The reference (ImanolGo/murmuration-kernels) exposes its GPU step only as an
 * executable contract: `flock_cuda --in F [--steps K] [--warmup W] [--out F]`
 * reading and writing the FLK1 state file (cuda/flock.cu:374-523,
 * crates/flock-ref/src/state.rs:104-171). Each entry point below replaces one
 * piece of that program, so a host in any language (the reference's Rust
 * crates through a thin FFI, Python through ctypes, the bundled CLI) can drive
 * the step in-process. Plain pointers and sizes only; no CUDA or torch types.
 *
 * State words: a flock of n birds is n*15 little-endian 4-byte words in the
 * .flk record order (state.rs:1-7): pos xyz, vel xyz, roll, spin, radius,
 * steering xyz, next_decision, neighbour count (u32 bits), centrality.
 *
 * Conventions: every call returns FLK_OK (0) or a negative FLK_ERR_* code and
 * never exits the process; flk_last_error() gives the calling thread's last
 * message. The library owns device memory; the caller owns host buffers and
 * states are copied in and out. A flock handle is used by one thread at a
 * time; a pool is internally synchronised. Device-side failures (a scan wait
 * that gave up) surface as FLK_ERR_DEVICE from the call that ran the step.
 */
#ifndef FLOCK_GB300_H
#define FLOCK_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FLK_OK 0
#define FLK_ERR_ARG -1      /* bad argument (null pointer, size) */
#define FLK_ERR_IO -2       /* file open/read/write failed, truncated file */
#define FLK_ERR_CUDA -3     /* a CUDA runtime call failed */
#define FLK_ERR_ID -4       /* unknown flock id or ticket */
#define FLK_ERR_CAPACITY -5 /* a batch exceeds the index space */
#define FLK_ERR_DEVICE -6   /* the device error word was set during a step */
#define FLK_ERR_FORMAT -7   /* not a FLK1 file with 15 words per bird */
#define FLK_ERR_BUDGET -8   /* request can never fit the pool's memory budget */

#define FLK_WORDS 15

/* ---- plain single-flock step (the drop-in for flock_cuda) ---------------- */
typedef struct flk_flock flk_flock;

/* Mean GPU ms per pass over the timed steps, the reference's stdout table
 * (cuda/flock.cu:474-492): hash+count, scan, scatter+sort, decide, integrate. */
typedef struct {
    double hash_ms, scan_ms, sort_ms, decide_ms, integrate_ms, total_ms;
    int32_t timed_steps;
} flk_pass_times;

/* Uploads a flock from host words (replaces read_flk + the H2D copies,
 * cuda/flock.cu:391,414-437). device < 0 uses the current device. */
int flk_open_host(int32_t device, uint32_t n, float time, const float* words, flk_flock** out);
/* Reads a .flk file and uploads it (cuda/flock.cu:340-354). */
int flk_open_file(int32_t device, const char* path, flk_flock** out);
/* Advances `steps` steps (the step loop, cuda/flock.cu:453-470); returns
 * after the work is queued and checked (synchronises). */
int flk_step(flk_flock* f, uint32_t steps);
/* Same, launched pass by pass with CUDA events; fills the per-pass means of
 * the last steps-warmup steps (cuda/flock.cu:447-492). */
int flk_step_timed(flk_flock* f, uint32_t steps, uint32_t warmup, flk_pass_times* out);
/* Copies the state back (replaces the D2H copies, cuda/flock.cu:494-519). */
int flk_read_host(flk_flock* f, float* time, float* words);
/* Writes the state as a .flk file (cuda/flock.cu:356-364). */
int flk_write_file(flk_flock* f, const char* path);
/* Bird count and canonical bucket count (cuda/flock.cu:368-372). */
int flk_size(const flk_flock* f, uint32_t* n, uint32_t* buckets);
/* The reference's decide occupancy experiment (--decide-smem N and the
 * "# decide occupancy" line, cuda/flock.cu:377,385,440-445): reserves
 * `extra_smem` bytes of dynamic shared memory per decide CTA beyond what
 * decide uses itself (0 = none), for every later step of this flock, and
 * reports the resulting launch: resident CTAs per SM, threads per CTA, the
 * SM's thread limit and the CTA's dynamic shared memory in bytes. Any output
 * may be NULL. A reservation no CTA can hold is FLK_ERR_ARG. */
int flk_decide_occupancy(flk_flock* f, uint64_t extra_smem, int32_t* blocks_per_sm, int32_t* threads,
                         int32_t* threads_per_sm, uint64_t* smem_bytes);
/* Runs ONE step and returns the grid it built and the neighbour-set summary
 * of every deciding bird, for bit-exact parity checks:
 *   keys[n]          bucket of each bird (cuda/flock.cu:118-124 grid_histogram)
 *   offsets[B+1]     exclusive scan of the bucket counts (grid_scan_*)
 *   sorted[n]        birds in (bucket, bird index) order (grid_scatter, made stable)
 *   sets[8n]         per bird: n_all, n_star, n_align, n_g and a wrapping sum of
 *                    mix(j) over each of those sets (model.rs:67-115); zeros for
 *                    birds that did not decide.
 * Any output pointer may be NULL. */
int flk_step_debug(flk_flock* f, uint32_t* keys, uint32_t* offsets, uint32_t* sorted, uint32_t* sets);
/* Cumulative deciding birds, candidate tests and pairs within 2R (counters of
 * the decide pass, cuda/flock.cu:190-290; the reference keeps none). */
int flk_counters(flk_flock* f, uint64_t* due, uint64_t* candidates, uint64_t* pairs);
/* One step (exactly flk_step(f, 1)) that also evaluates the same step in FP64
 * from the same input state, for error reports on a live flock. `out64`
 * (optional, n*15 doubles, bird order) receives the FP64 post-step state;
 * `report` (optional, 4 doubles) the f32 step's maximum relative position
 * error, maximum relative velocity error, neighbour-count mismatches and the
 * number of deciding birds. The reference evaluates only in f32; its oracle
 * (crates/flock-ref/src/model.rs:53-176) is what the FP64 pass restates. */
int flk_step_f64(flk_flock* f, double* out64, double* report);
/* Measurement helper (no counterpart in the reference, whose main() times
 * passes inline, cuda/flock.cu:447-492): runs `steps` steps one graph launch
 * at a time; before each step it overwrites a `flush_bytes` device buffer so
 * the step starts with a cold L2, then brackets the step with CUDA events on
 * the library's stream. ms_per_step[steps] receives each step's device time.
 * Each step runs as in flk_step's multi-step runs: its integrate also counts
 * the next step's grid. The first grid is counted before the first timed step
 * and one untimed step follows the last, so the flock advances steps + 1. */
int flk_time_steps(flk_flock* f, uint32_t steps, uint64_t flush_bytes, float* ms_per_step);
/* flk_batch_tune_cell for a plain flock. */
int flk_tune_cell(flk_flock* f, float cell_m);
/* flk_batch_tune_decide for a plain flock. */
int flk_tune_decide(flk_flock* f, int32_t staged);
/* Frees the flock's device memory (the cudaFree calls closing main,
 * cuda/flock.cu:520-523). */
void flk_close(flk_flock* f);

/* ---- batched: many independent flocks, one launch per pass --------------- */
/* No counterpart in the reference, whose backends run one flock per process
 * (cuda/flock.cu:374-523). Each flock of a batch steps exactly as the plain
 * step would step it alone; the calls below mirror the plain ones. */
typedef struct flk_batch flk_batch;

/* An empty batch on `device` (< 0: the current device); no counterpart. */
int flk_batch_create(int32_t device, flk_batch** out);
/* Adds a flock (as flk_open_host); *id receives its handle within the batch. */
int flk_batch_add(flk_batch* b, uint32_t n, float time, const float* words, int32_t* id);
/* Drops a flock and frees its storage for later flocks; no counterpart. */
int flk_batch_remove(flk_batch* b, int32_t id);
/* Advances every flock in the batch by `steps` steps (10-step CUDA graphs). */
int flk_batch_step(flk_batch* b, uint32_t steps);
/* Steps only the listed flocks, each by its own count (0 = idle). */
int flk_batch_step_each(flk_batch* b, const int32_t* ids, const uint32_t* steps, uint32_t count);
/* One flock's state, as flk_read_host (cuda/flock.cu:494-519). */
int flk_batch_read(flk_batch* b, int32_t id, float* time, float* words);
/* One step of every flock; per-flock grid/sets outputs concatenated in id
 * order of `ids` (same layouts as flk_step_debug, offsets per flock B_f+1). */
int flk_batch_step_debug(flk_batch* b, const int32_t* ids, uint32_t count, uint32_t* keys, uint32_t* offsets,
                         uint32_t* sorted, uint32_t* sets);
/* flk_step_f64 for the listed flocks (one step each, the others idle):
 * `out64` (optional) receives each listed flock's FP64 post-step state
 * (n_f*15 doubles, bird order) concatenated in the order of `ids`; `reports`
 * (optional, 4 doubles per id) each flock's own error report, as flk_step_f64
 * gives it. A duplicated id is FLK_ERR_ARG. */
int flk_batch_step_f64(flk_batch* b, const int32_t* ids, uint32_t count, double* out64, double* reports);
/* Launch shape: CTAs per SM of the streaming passes and decide, decide CTA
 * size, steps per captured graph. Zero keeps the current value. No
 * counterpart: the reference fixes its launch shapes (cuda/flock.cu:453-470). */
int flk_batch_tune(flk_batch* b, int32_t stream_bps, int32_t decide_bps, int32_t decide_threads, int32_t graph_chunk);
/* Production cell edge in metres (default 4 m, the reference's; [2, 16],
 * else FLK_ERR_ARG): the cells that steps without grid output sort birds
 * into, in quarter-cell z-slabs, and search. It changes which candidates
 * decide tests, never which neighbours it finds (exact distance tests decide
 * membership); sums may change by rounding. Grid-reporting steps
 * (flk_step_debug) always use the reference's 4 m cells
 * (crates/flock-ref/src/params.rs:58, cuda/flock.cu:77-83). No counterpart:
 * the reference's cell is a compile-time constant. */
int flk_batch_tune_cell(flk_batch* b, float cell_m);
/* Which decide kernel steps without grid output run (0, the default, sweeps
 * the cell-ordered state through the caches; 1 stages each CTA's
 * neighbourhood in shared memory with TMA bulk copies first, falling back to
 * the direct sweep where birds of several flocks meet). Both find the same
 * neighbours and give the same decisions; sums may differ by rounding. Other
 * values: FLK_ERR_ARG. No counterpart: the reference's decide
 * (cuda/flock.cu:190-290) reads every candidate from global memory. */
int flk_batch_tune_decide(flk_batch* b, int32_t staged);
/* Chunk graphs instantiated, and updated in place (cudaGraphExecUpdate, when
 * only sizes or pointers changed, e.g. a flock joined or left), so far. */
int flk_batch_graph_counts(flk_batch* b, uint64_t* instantiated, uint64_t* updated);
/* flk_counters summed over the batch's flocks. */
int flk_batch_counters(flk_batch* b, uint64_t* due, uint64_t* candidates, uint64_t* pairs);
/* Times `steps` graph-launched steps on the batch's stream with CUDA events. */
int flk_batch_time_steps(flk_batch* b, uint32_t steps, double* ms);
/* Every flock of the batch, `steps` eager steps with per-pass events; means of
 * the last steps-warmup steps (as flk_step_timed). */
int flk_batch_step_timed(flk_batch* b, uint32_t steps, uint32_t warmup, flk_pass_times* out);
/* Frees the batch and all its flocks (as flk_close). */
void flk_batch_destroy(flk_batch* b);

/* ---- served: continuous batching of simulate(flock, steps) requests ------ */
/* No counterpart in the reference (one flock per process, cuda/flock.cu:374-523):
 * requests arrive while others run, join the batched step at chunk boundaries
 * and leave it when done; each result equals the plain step's alone. */
typedef struct flk_pool flk_pool;

typedef struct {
    uint64_t submitted, completed, rejected;
    uint64_t bird_steps;     /* sum of n * steps over completed requests */
    uint64_t resident_bytes; /* device bytes held by admitted flocks */
    uint64_t chunks;         /* batched chunks run */
    double busy_ms;          /* wall time the worker spent with work in flight */
} flk_pool_stats;

/* A worker thread owns the device; `budget_bytes` caps the device memory of
 * admitted flocks; arrivals join the batch at chunk boundaries every
 * `chunk_steps` steps. */
int flk_pool_create(int32_t device, uint64_t budget_bytes, uint32_t chunk_steps, flk_pool** out);
/* Queues simulate(flock, steps). `words` must stay valid until the request
 * completes; the result (and its clock) are written to `out_words` /
 * `out_time`, which may alias the input. */
int flk_pool_submit(flk_pool* p, uint32_t n, float time, const float* words, uint32_t steps, float* out_words,
                    float* out_time, uint64_t* ticket);
/* flk_pool_submit with the state read from a .flk file (state.rs:104-171);
 * the pool holds its own copy of the input. The result buffer must hold
 * `out_capacity` birds; *n_out receives the flock's size (flk_file_info reads
 * it beforehand). No counterpart in the reference, whose tools read a file
 * per process (cuda/flock.cu:340-354). */
int flk_pool_submit_file(flk_pool* p, const char* path, uint32_t steps, float* out_words, uint32_t out_capacity,
                         float* out_time, uint64_t* ticket, uint32_t* n_out);
/* Copies a request's current state into `words` (n*15 words) without pausing
 * the other flocks: a queued request gives its input (0 steps done), a
 * resident one its state at the next chunk boundary (packed on the compute
 * stream, copied on the copy stream while the next chunk runs), a finished
 * one its result. Blocks until the copy has landed. With `path`, also writes
 * the state as a .flk file, so submitting that file with the remaining steps
 * continues the flock exactly. No counterpart in the reference. */
int flk_pool_snapshot(flk_pool* p, uint64_t ticket, float* words, float* time, uint32_t* steps_done,
                      const char* path);
/* Error report of a request's next step: takes the request's current state
 * as flk_pool_snapshot does (steps_done optional), then runs flk_step_f64 on
 * a private copy on the pool's device. The served flock is not advanced;
 * `out64` (optional, n*15) and `report` (optional, 4) as in flk_step_f64.
 * The copy's device memory is outside the pool's budget. */
int flk_pool_error_report(flk_pool* p, uint64_t ticket, double* out64, double* report, uint32_t* steps_done);
/* *state: 0 queued, 1 resident, 2 done, negative FLK_ERR_* on failure. */
int flk_pool_poll(flk_pool* p, uint64_t ticket, int32_t* state);
/* Blocks until done; *latency_ms = completion - submission (host clock). */
int flk_pool_wait(flk_pool* p, uint64_t ticket, double* latency_ms);
/* Counters since creation (the struct above). */
int flk_pool_stats_get(flk_pool* p, flk_pool_stats* out);
/* Stops the worker and frees the pool. Results already being copied out land
 * first; requests still queued or resident are dropped (their output buffers
 * are not written). No other call on the pool may be in progress or follow. */
void flk_pool_destroy(flk_pool* p);

/* ---- failure paths ------------------------------------------------------- */
/* Text for a device error word (what FLK_ERR_DEVICE's message reports):
 * 1 = a scan look-back wait gave up, 2 = a bucket range or slot fell outside
 * its array and was skipped. The reference has no device error word: its CK
 * macro prints and exits (cuda/flock.cu:27-34). */
const char* flk_device_error_text(uint32_t word);
/* Test hook for the bounded device waits; no counterpart. Arms the flock's
 * NEXT grid-reporting step (flk_step_debug): scan tile `skip_tile` publishes
 * no look-back flag, so the tiles after it wait for a flag nothing sets, and
 * every look-back gives up after `spin_limit` polls (0 keeps the usual limit
 * of 2^22). That step returns FLK_ERR_DEVICE with the scan-timeout text and
 * leaves the flock's state unusable (close it); the device and the process
 * stay usable. No fault, trap or unbounded wait is involved. */
int flk_debug_scan_timeout(flk_flock* f, uint32_t skip_tile, uint32_t spin_limit);

/* ---- helpers -------------------------------------------------------------- */
/* The calling thread's last error message: what the CK macro prints before
 * exit(1) (cuda/flock.cu:27-34), returned instead. */
const char* flk_last_error(void);
/* Bird count and clock from a .flk header (state.rs:104-171). */
int flk_file_info(const char* path, uint32_t* n, float* time);
/* Canonical bucket count: next power of two >= 2n clamped to [2^16, 2^22]
 * (cuda/flock.cu:368-372). */
uint32_t flk_buckets_for(uint32_t n);
/* The benchmark scatter (state.rs:79-101): n birds, SplitMix64 seed. */
int flk_generate(uint32_t n, uint64_t seed, float* words);
/* Model constants in the order DT, DU, V0, MASS, CL_CD, G, L0, D0, TAU,
 * TAU_ROLL, MAX_ROLL_RATE, MAX_BANK, V_MIN, V_MAX, N_C, R_MAX, RADIUS_LERP,
 * R_H, SIGMA, W_SEP, W_ALIGN, W_COH, BLIND_COS, W_ROOST_V, H_ROOST_V, Z0,
 * GRID_CELL, RADIUS_EXP (params.rs:5-65). Returns the count written. */
int flk_params(float* out, int32_t cap);
/* Device bytes a flock of n birds occupies when resident (the pool's admission
 * unit); no counterpart. */
uint64_t flk_bytes_for(uint32_t n);
/* Engine kernel launches per step (for launch accounting); the reference's
 * step launches seven (cuda/flock.cu:453-470). */
int flk_kernels_per_step(void);
/* Page-locks / releases a caller's host buffer so state copies run at full
 * link speed (cudaHostRegister / cudaHostUnregister); no counterpart (the
 * reference copies from pageable vectors, cuda/flock.cu:414-437). */
int flk_pin(void* ptr, uint64_t bytes);
int flk_unpin(void* ptr);

/* ---- grid build without device allocation ------------------------------- */
/* No counterpart in the reference. For callers that may not allocate device
 * memory themselves or let a library do it: a host that manages all device
 * memory through its own pool, a real-time loop that cannot afford
 * cudaMalloc's implicit synchronisation, a plugin with a fixed memory budget.
 * Builds one flock's grid -- the same keys[n], offsets[buckets_for(n)+1] and
 * stable sorted[n] that flk_step_debug reports -- from n positions
 * pos4[4n] (x, y, z, unused) in device memory into caller-owned device
 * buffers (pos4 and offsets 16-byte aligned), on `stream` (a cudaStream_t,
 * NULL = legacy default stream). It is a blocking call: it synchronises that
 * stream before returning, so it cannot run under stream capture or inside a
 * CUDA graph. It calls no allocator: its
 * scratch is one fixed device array inside the library (about 2.5 MiB, held on
 * every GPU that loads the library until exit), sized for at most
 * FLK_NOALLOC_MAX_BIRDS birds; larger n returns FLK_ERR_CAPACITY. Each call
 * looks up that array's device address on the current device. n = 0 still
 * writes all buckets_for(0)+1 = 65,537 offsets (zeros). Calls share the array:
 * concurrent calls on one device race. */
#define FLK_NOALLOC_MAX_BIRDS 131072u
int flk_grid_noalloc(const float* pos4, uint32_t n, uint32_t* keys, uint32_t* offsets, uint32_t* sorted, void* stream);

#ifdef __cplusplus
}
#endif
#endif
