/*
 * flock_oracle.h -- CPU oracle for the starling-flock step.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker: a plain-C restatement of the
 * reference's Rust CPU oracle (crates/flock-ref). Only tests/, the smoke check
 * in __graft_entry__.py and bench.py's CPU-baseline / reference arm may load
 * it. The product (murmuration_kernels_gb300) never links or calls it.
 *
 * What it restates (file:line in the reference project):
 *   constants            crates/flock-ref/src/params.rs:5-58
 *   radius_step          crates/flock-ref/src/params.rs:61-65
 *   Bird / Flock / .flk  crates/flock-ref/src/state.rs:16-49, 104-171
 *   SplitMix64, scatter  crates/flock-ref/src/state.rs:58-101
 *   forward/side/up      crates/flock-ref/src/model.rs:15-38
 *   decide               crates/flock-ref/src/model.rs:53-145
 *   step_bird            crates/flock-ref/src/model.rs:149-176
 *   Flock::step          crates/flock-ref/src/model.rs:182-200
 *   stats/statdiff/diff  crates/flock-ref/src/main.rs:83-208
 *   grid keys / buckets  cuda/flock.cu:75-83, 368-372
 *   grid invariants      cutile/src/main.rs:307-362 (check_grid)
 *   CPU grid step        cuda/flock.cu:85-91, 190-290 (orc_step_grid, a baseline)
 *
 * Vector arithmetic follows glam 0.34.1's scalar Vec3 (the reference's
 * Cargo.lock:219-221; glam is not vendored): component-wise f32 operations,
 * dot = (x*x' + y*y') + z*z' left to right, normalize = v * (1/length),
 * normalize_or_zero = zero unless 1/length is finite and > 0, Vec3 / s is a
 * component-wise division. Every expression is evaluated in f32 with no FMA
 * contraction (the build passes -ffp-contract=off); transcendentals come from
 * the host libm, as Rust's f32 methods do.
 *
 * Parity pins: the reference's own unit tests (state.rs:177-197,
 * model.rs:208-269) are restated in tests/test_oracle.py, and the oracle is
 * checked against fixtures produced by the reference's own CUDA kernels
 * (cuda/flock.cu, built unchanged for sm_103a) under tests/golden/.
 */
#ifndef FLOCK_ORACLE_H
#define FLOCK_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One bird record, exactly the 15 little-endian words of a .flk record
 * (state.rs:1-7): pos xyz, vel xyz, roll, spin, radius, steering xyz,
 * next_decision, neighbour count (u32), centrality. */
typedef struct {
    float pos[3];
    float vel[3];
    float roll;
    float spin;
    float radius;
    float steer[3];
    float next_decision;
    uint32_t neighbours;
    float centrality;
} orc_bird;

/* Per-decision set summary used to compare neighbour sets bit for bit without
 * storing them: counts of the four sets decide() forms, plus an
 * order-independent hash of each (wrapping sum of orc_set_mix(j)). */
typedef struct {
    uint32_t n_all, n_star, n_align, n_g;
    uint32_t h_all, h_star, h_align, h_g;
} orc_sets;

typedef struct {
    float force[3];
    float radius;
    uint32_t neighbours;
    float centrality;
} orc_decision;

/* Constants as f32 values (params.rs), exported so tests can compare them
 * with the product's copy word for word. Order: see orc_param_names. */
enum { ORC_NPARAMS = 28 };
void orc_params(float out[ORC_NPARAMS]);
const char* orc_param_name(int k);

uint32_t orc_set_mix(uint32_t j);
float orc_radius_step(float r, uint32_t n);

/* state.rs:79-101. Writes n birds; returns the world time (0). */
void orc_scatter(uint32_t n, uint64_t seed, orc_bird* out);
/* state.rs:104-171: returns 0, or -1 bad magic / words, -2 truncated / IO. */
int orc_write_flk(const char* path, float time, const orc_bird* b, uint32_t n);
int orc_read_header(const char* path, uint32_t* n, float* time);
int orc_read_flk(const char* path, float* time, orc_bird* out, uint32_t n);

/* model.rs:53-145 for bird i over a snapshot of all n birds. `sets` may be NULL. */
orc_decision orc_decide(uint32_t i, const orc_bird* birds, uint32_t n, float z0, orc_sets* sets);
/* model.rs:149-176. */
void orc_step_bird(orc_bird* b, float dt);
/* model.rs:182-200: one step in place. `sets_out` (n entries, may be NULL)
 * receives the set summary of each deciding bird (zeros for the others);
 * `due_out` (may be NULL) receives 1 for deciding birds. `threads` <= 0 uses
 * the OpenMP default. Returns the new time. */
float orc_step(orc_bird* birds, uint32_t n, float time, orc_sets* sets_out, uint8_t* due_out, int threads);
/* FP64 evaluation of one step from the same f32 input (same formulas in
 * double; set membership tested in double too). Writes doubles in .flk word
 * order (15 per bird; word 13 holds the neighbour count). */
double orc_step_f64(const orc_bird* birds, uint32_t n, float time, double* out_words, int threads);

/* CPU-baseline sample: decide() for birds idx[0..m) against all n (OpenMP),
 * results discarded into a checksum. Returns the checksum. */
double orc_decide_sample(const orc_bird* birds, uint32_t n, const uint32_t* idx, uint32_t m, int threads);
/* decide() for birds idx[0..m) against all n birds (OpenMP): decisions and
 * set summaries per listed bird (either output may be NULL). */
void orc_decide_many(const orc_bird* birds, uint32_t n, const uint32_t* idx, uint32_t m, orc_sets* sets,
                     orc_decision* out, int threads);
/* step_bird for all n birds (OpenMP). */
void orc_integrate_all(orc_bird* birds, uint32_t n, int threads);

/* Grid restatement (cuda/flock.cu:75-83, 368-372) with the canonical stable
 * order (bucket, then bird index). keys: n, offsets: buckets+1, sorted: n. */
/* One step with the reference GPU backend's grid algorithm (cuda/flock.cu:
 * 190-290: R and 2R cell walks with the exact cell check) run on host cores;
 * a CPU baseline, checked against orc_step. Returns the new time. */
float orc_step_grid(orc_bird* birds, uint32_t n, float time, int threads);

uint32_t orc_buckets_for(uint32_t n);
void orc_cell_of(const float p[3], int32_t c[3]);
uint32_t orc_bucket_of(const int32_t c[3], uint32_t mask);
void orc_grid(const orc_bird* birds, uint32_t n, uint32_t buckets, uint32_t* keys, uint32_t* offsets, uint32_t* sorted);
/* cutile/src/main.rs:307-362 invariants. 0 = ok, else a code naming the failure. */
int orc_check_grid(const uint32_t* keys, const uint32_t* offsets, const uint32_t* sorted, uint32_t n, uint32_t buckets,
                   const orc_bird* birds);

/* main.rs:83-90: mean speed, mean neighbours, mean radius, polarization. */
void orc_stats(const orc_bird* b, uint32_t n, float out[4]);
/* main.rs:136-208. Fills out[0..7) = max |dpos|, |dvel|, |dradius|,
 * |dcentrality|, |dsteering|, |droll|, |dspin|; *mismatch = neighbour-count
 * mismatches; *outliers = birds above pos_tol/vel_tol. Returns 1 on PASS. */
int orc_diff(const orc_bird* a, const orc_bird* b, uint32_t n, float pos_tol, float vel_tol, uint32_t allow,
             float outlier_max, float out[7], uint32_t* mismatch, uint32_t* outliers);
/* main.rs:104-133. Returns 1 on PASS; out[0..4) = |d| of the four stats. */
int orc_statdiff(const orc_bird* a, const orc_bird* b, uint32_t n, float out[4]);

int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
