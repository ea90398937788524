/*
 * flock_oracle.c -- CPU oracle for the starling-flock step (test infrastructure).
 *
 * A plain-C restatement of the reference's Rust oracle, expression by
 * expression; see flock_oracle.h for the file:line map and the glam
 * assumptions. Build with -ffp-contract=off (no FMA contraction) and without
 * -ffast-math so every f32 operation rounds exactly as rustc's does.
 */
#include "flock_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- constants: crates/flock-ref/src/params.rs:5-58 (f32 folding) ------- */
#define P_DT 0.005f
#define P_DU 0.05f
#define P_V0 10.0f
#define P_MASS 0.08f
#define P_CL_CD 3.3f
#define P_G 9.81f
static const float P_L0 = P_MASS * P_G;
static const float P_D0 = (P_MASS * P_G) / P_CL_CD;
#define P_TAU 1.0f
#define P_TAU_ROLL 0.15f
#define P_MAX_ROLL_RATE 6.0f
static const float P_MAX_BANK = 80.0f * 3.14159265358979323846f / 180.0f;
static const float P_V_MIN = 0.5f * P_V0;
static const float P_V_MAX = 2.0f * P_V0;
#define P_N_C 6.5f
#define P_R_MAX 100.0f
#define P_RADIUS_LERP 0.1f
#define P_R_H 0.2f
#define P_SIGMA 1.37f
#define P_W_SEP 1.0f
#define P_W_ALIGN 0.5f
#define P_W_COH 0.65f
static const float P_BLIND_COS = -0.70710678118654752440f;
#define P_W_ROOST_V 0.2f
#define P_H_ROOST_V 40.0f
#define P_Z0 100.0f
#define P_GRID_CELL 4.0f
static const float P_RADIUS_EXP = P_RADIUS_LERP / 3.0f;
/* state.rs:52-54 */
#define P_DENSITY 0.5f
#define P_START_RADIUS 1.5f

static const char* const k_param_names[ORC_NPARAMS] = {
    "DT",   "DU",      "V0",        "MASS",    "CL_CD",       "G",         "L0",          "D0",        "TAU",   "TAU_ROLL",
    "MAX_ROLL_RATE", "MAX_BANK", "V_MIN", "V_MAX", "N_C", "R_MAX", "RADIUS_LERP", "R_H", "SIGMA", "W_SEP",
    "W_ALIGN", "W_COH", "BLIND_COS", "W_ROOST_V", "H_ROOST_V", "Z0", "GRID_CELL", "RADIUS_EXP"};

void orc_params(float out[ORC_NPARAMS]) {
    const float v[ORC_NPARAMS] = {P_DT,        P_DU,      P_V0,        P_MASS,      P_CL_CD,      P_G,
                                  P_L0,        P_D0,      P_TAU,       P_TAU_ROLL,  P_MAX_ROLL_RATE, P_MAX_BANK,
                                  P_V_MIN,     P_V_MAX,   P_N_C,       P_R_MAX,     P_RADIUS_LERP, P_R_H,
                                  P_SIGMA,     P_W_SEP,   P_W_ALIGN,   P_W_COH,     P_BLIND_COS,  P_W_ROOST_V,
                                  P_H_ROOST_V, P_Z0,      P_GRID_CELL, P_RADIUS_EXP};
    memcpy(out, v, sizeof v);
}

const char* orc_param_name(int k) { return (k >= 0 && k < ORC_NPARAMS) ? k_param_names[k] : NULL; }

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---- glam Vec3 (scalar) -------------------------------------------------- */
typedef struct { float x, y, z; } v3;

static inline v3 V(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 v_add(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 v_sub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 v_mul(v3 a, float s) { return V(a.x * s, a.y * s, a.z * s); }
static inline v3 v_div(v3 a, float s) { return V(a.x / s, a.y / s, a.z / s); }
static inline float v_dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 v_cross(v3 a, v3 b) {
    return V(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
static inline float v_len(v3 a) { return sqrtf(v_dot(a, a)); }
static inline v3 v_normalize(v3 a) { return v_mul(a, 1.0f / v_len(a)); }
static inline v3 v_normalize_or_zero(v3 a) {
    float rcp = 1.0f / v_len(a);
    return (isfinite(rcp) && rcp > 0.0f) ? v_mul(a, rcp) : V(0.0f, 0.0f, 0.0f);
}
static inline float f_max(float a, float b) { return fmaxf(a, b); }
/* f32::clamp: NaN passes through. */
static inline float f_clamp(float v, float lo, float hi) {
    if (v < lo) v = lo;
    if (v > hi) v = hi;
    return v;
}
static const v3 VX = {1.0f, 0.0f, 0.0f};
static const v3 VZ = {0.0f, 0.0f, 1.0f};
static const v3 V0V = {0.0f, 0.0f, 0.0f};

static inline v3 pos_of(const orc_bird* b) { return V(b->pos[0], b->pos[1], b->pos[2]); }
static inline v3 vel_of(const orc_bird* b) { return V(b->vel[0], b->vel[1], b->vel[2]); }

/* ---- params.rs:61-65 ----------------------------------------------------- */
float orc_radius_step(float r, uint32_t n) {
    float nn = (float)(n > 1u ? n : 1u);
    float factor = powf(P_N_C / nn, P_RADIUS_EXP);
    return f_clamp(r * factor, P_R_H, P_R_MAX);
}

/* Order-independent set hash term (a murmur3-style 32-bit finaliser of j+1). */
uint32_t orc_set_mix(uint32_t j) {
    uint32_t h = j + 1u;
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

/* ---- state.rs:58-101 ------------------------------------------------------ */
typedef struct { uint64_t s; } splitmix;
static uint64_t sm_next(splitmix* r) {
    r->s += 0x9E3779B97F4A7C15ull;
    uint64_t z = r->s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static float sm_unit(splitmix* r) { return (float)(sm_next(r) >> 40) / (float)(1ull << 24); }

void orc_scatter(uint32_t n, uint64_t seed, orc_bird* out) {
    const float side = cbrtf((float)n / P_DENSITY);
    const v3 centre = V(0.0f, 0.0f, P_Z0);
    splitmix rng = {seed};
    for (uint32_t i = 0; i < n; ++i) {
        float ox = (sm_unit(&rng) - 0.5f) * side;
        float oy = (sm_unit(&rng) - 0.5f) * side;
        float oz = (sm_unit(&rng) - 0.5f) * side;
        float jx = sm_unit(&rng) - 0.5f;
        float jy = sm_unit(&rng) - 0.5f;
        float jz = sm_unit(&rng) - 0.5f;
        v3 jitter = v_mul(V(jx, jy, jz), 0.05f);
        v3 pos = v_add(centre, V(ox, oy, oz));
        v3 vel = v_mul(v_normalize(v_add(VX, jitter)), P_V0);
        orc_bird b;
        memset(&b, 0, sizeof b);
        b.pos[0] = pos.x; b.pos[1] = pos.y; b.pos[2] = pos.z;
        b.vel[0] = vel.x; b.vel[1] = vel.y; b.vel[2] = vel.z;
        b.radius = P_START_RADIUS;
        b.next_decision = sm_unit(&rng) * P_DU;
        out[i] = b;
    }
}

/* ---- state.rs:104-171: the .flk file -------------------------------------- */
int orc_write_flk(const char* path, float time, const orc_bird* b, uint32_t n) {
    FILE* fp = fopen(path, "wb");
    if (!fp) return -2;
    uint32_t head[4] = {0x314B4C46u, n, 15u, 0u};
    memcpy(&head[3], &time, 4);
    int ok = fwrite(head, 4, 4, fp) == 4 && (n == 0 || fwrite(b, sizeof(orc_bird), n, fp) == n);
    ok &= fclose(fp) == 0;
    return ok ? 0 : -2;
}

int orc_read_header(const char* path, uint32_t* n, float* time) {
    FILE* fp = fopen(path, "rb");
    if (!fp) return -2;
    uint32_t head[4];
    size_t got = fread(head, 4, 4, fp);
    fclose(fp);
    if (got != 4) return -2;
    if (memcmp(head, "FLK1", 4) != 0 || head[2] != 15u) return -1;
    *n = head[1];
    memcpy(time, &head[3], 4);
    return 0;
}

int orc_read_flk(const char* path, float* time, orc_bird* out, uint32_t n) {
    uint32_t hn;
    int rc = orc_read_header(path, &hn, time);
    if (rc) return rc;
    if (hn != n) return -1;
    FILE* fp = fopen(path, "rb");
    if (!fp) return -2;
    fseek(fp, 16, SEEK_SET);
    size_t got = n ? fread(out, sizeof(orc_bird), n, fp) : 0;
    fclose(fp);
    return got == n ? 0 : -2;
}

/* ---- model.rs:15-38 ------------------------------------------------------- */
static inline v3 forward(v3 v) { return v_dot(v, v) > 1e-12f ? v_normalize(v) : VX; }
static inline v3 side_of(v3 f) {
    v3 s = v_cross(f, VZ);
    return v_dot(s, s) > 1e-8f ? v_normalize(s) : VX;
}
static inline v3 body_up(v3 f, float beta) {
    v3 side = side_of(f);
    v3 up0 = v_cross(side, f);
    return v_add(v_mul(up0, cosf(beta)), v_mul(side, sinf(beta)));
}

/* ---- model.rs:53-145 ------------------------------------------------------ */
orc_decision orc_decide(uint32_t i, const orc_bird* birds, uint32_t n, float z0, orc_sets* sets) {
    const orc_bird* me = &birds[i];
    const v3 p = pos_of(me);
    const float r = me->radius;
    const v3 f_i = forward(vel_of(me));

    v3 sep = V0V, coh = V0V, align = V0V;
    uint32_t n_all = 0, n_star = 0, n_align = 0;
    uint32_t h_all = 0, h_star = 0, h_align = 0, h_g = 0;

    const float r2 = r * r;
    for (uint32_t j = 0; j < n; ++j) {
        if (j == i) continue;
        const v3 d = v_sub(pos_of(&birds[j]), p);
        const float d2 = v_dot(d, d);
        if (d2 > r2) continue;
        const float dist = sqrtf(d2);
        n_all += 1;
        h_all += orc_set_mix(j);
        const v3 dhat = v_div(d, f_max(dist, 1e-6f));
        float g;
        if (dist <= P_R_H) {
            g = 1.0f;
        } else {
            const float t = dist - P_R_H;
            g = expf(-(t * t) / (2.0f * P_SIGMA * P_SIGMA));
        }
        sep = v_sub(sep, v_mul(dhat, g));
        if (dist > P_R_H) {
            coh = v_add(coh, dhat);
            n_star += 1;
            h_star += orc_set_mix(j);
        }
        if (v_dot(f_i, dhat) >= P_BLIND_COS) {
            align = v_add(align, forward(vel_of(&birds[j])));
            n_align += 1;
            h_align += orc_set_mix(j);
        }
    }

    v3 force = V0V;
    if (n_all > 0) force = v_add(force, v_mul(sep, P_W_SEP / (float)n_all));

    /* Centrality over 2R_i (Eq. 7). */
    const float c2 = (2.0f * r) * (2.0f * r);
    v3 csum = V0V;
    uint32_t n_g = 0;
    for (uint32_t j = 0; j < n; ++j) {
        if (j == i) continue;
        const v3 d = v_sub(pos_of(&birds[j]), p);
        const float d2 = v_dot(d, d);
        if (d2 > c2) continue;
        csum = v_add(csum, v_div(d, f_max(sqrtf(d2), 1e-6f)));
        n_g += 1;
        h_g += orc_set_mix(j);
    }
    const float centrality = n_g > 0 ? v_len(csum) / (float)n_g : 0.0f;

    if (n_star > 0) force = v_add(force, v_mul(v_normalize_or_zero(coh), P_W_COH * centrality));
    const v3 a = n_align > 0 ? v_sub(v_div(align, (float)n_align), f_i) : V0V;
    force = v_add(force, v_mul(a, P_W_ALIGN));

    /* Vertical roost pull (Eq. 12), capped. */
    force = v_add(force, v_mul(VZ, P_W_ROOST_V * f_clamp((z0 - p.z) / P_H_ROOST_V, -1.0f, 1.0f)));

    /* Speed control (Eq. 1). */
    const float speed = v_len(vel_of(me));
    force = v_add(force, v_mul(f_i, (P_MASS / P_TAU) * (P_V0 - speed)));

    if (sets) {
        sets->n_all = n_all; sets->n_star = n_star; sets->n_align = n_align; sets->n_g = n_g;
        sets->h_all = h_all; sets->h_star = h_star; sets->h_align = h_align; sets->h_g = h_g;
    }
    orc_decision out;
    out.force[0] = force.x; out.force[1] = force.y; out.force[2] = force.z;
    out.radius = orc_radius_step(r, n_all);
    out.neighbours = n_all;
    out.centrality = centrality;
    return out;
}

/* ---- model.rs:149-176 ----------------------------------------------------- */
void orc_step_bird(orc_bird* b, float dt) {
    v3 vel = vel_of(b);
    const v3 steering = V(b->steer[0], b->steer[1], b->steer[2]);
    const v3 f = forward(vel);
    const v3 side = side_of(f);
    const float speed = f_max(v_len(vel), 1e-6f);

    const float a_lat = v_dot(steering, side) / P_MASS;
    const float target = f_clamp(atanf(a_lat / P_G), -P_MAX_BANK, P_MAX_BANK);
    const float rate = f_clamp((target - b->roll) / P_TAU_ROLL, -P_MAX_ROLL_RATE, P_MAX_ROLL_RATE);
    b->spin = rate;
    const float beta = f_clamp(b->roll + rate * dt, -P_MAX_BANK, P_MAX_BANK);
    b->roll = beta;

    const v3 up = body_up(f, beta);
    const float cos_beta = f_max(cosf(beta), 0.2f);
    const float sr = speed / P_V0;
    const float lift = sr * sr * P_L0 / cos_beta;
    const float drag = sr * sr * P_D0;
    /* up*lift - f*drag + f*D0 - Z*MASS*G, left to right */
    const v3 flight = v_sub(v_add(v_sub(v_mul(up, lift), v_mul(f, drag)), v_mul(f, P_D0)), v_mul(v_mul(VZ, P_MASS), P_G));

    const v3 control = v_sub(steering, v_mul(side, v_dot(steering, side)));
    vel = v_add(vel, v_mul(v_div(v_add(control, flight), P_MASS), dt));
    const float sp = v_len(vel);
    if (sp > P_V_MAX) {
        vel = v_mul(vel, P_V_MAX / sp);
    } else if (sp < P_V_MIN && sp > 1e-6f) {
        vel = v_mul(vel, P_V_MIN / sp);
    }
    v3 pos = v_add(pos_of(b), v_mul(vel, dt));
    b->pos[0] = pos.x; b->pos[1] = pos.y; b->pos[2] = pos.z;
    b->vel[0] = vel.x; b->vel[1] = vel.y; b->vel[2] = vel.z;
}

/* ---- model.rs:182-200 ----------------------------------------------------- */
float orc_step(orc_bird* birds, uint32_t n, float time, orc_sets* sets_out, uint8_t* due_out, int threads) {
    time += P_DT;
    orc_decision* dec = (orc_decision*)malloc(sizeof(orc_decision) * (n ? n : 1));
    uint8_t* due = (uint8_t*)malloc(n ? n : 1);
    for (uint32_t i = 0; i < n; ++i) due[i] = time >= birds[i].next_decision;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads)
#endif
    for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
        uint32_t i = (uint32_t)ii;
        if (!due[i]) {
            if (sets_out) memset(&sets_out[i], 0, sizeof(orc_sets));
            continue;
        }
        dec[i] = orc_decide(i, birds, n, P_Z0, sets_out ? &sets_out[i] : NULL);
    }
    for (uint32_t i = 0; i < n; ++i) {
        if (!due[i]) continue;
        birds[i].steer[0] = dec[i].force[0];
        birds[i].steer[1] = dec[i].force[1];
        birds[i].steer[2] = dec[i].force[2];
        birds[i].radius = dec[i].radius;
        birds[i].neighbours = dec[i].neighbours;
        birds[i].centrality = dec[i].centrality;
        birds[i].next_decision += P_DU;
    }
    for (uint32_t i = 0; i < n; ++i) orc_step_bird(&birds[i], P_DT);
    if (due_out) memcpy(due_out, due, n);
    free(dec);
    free(due);
    (void)threads;
    return time;
}

double orc_decide_sample(const orc_bird* birds, uint32_t n, const uint32_t* idx, uint32_t m, int threads) {
    double acc = 0.0;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : acc) num_threads(threads)
#endif
    for (int64_t k = 0; k < (int64_t)m; ++k) {
        orc_decision d = orc_decide(idx[k], birds, n, P_Z0, NULL);
        acc += (double)d.force[0] + (double)d.radius + (double)d.neighbours;
    }
    (void)threads;
    return acc;
}

void orc_decide_many(const orc_bird* birds, uint32_t n, const uint32_t* idx, uint32_t m, orc_sets* sets,
                     orc_decision* out, int threads) {
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
    for (int64_t k = 0; k < (int64_t)m; ++k) {
        orc_sets s;
        orc_decision d = orc_decide(idx[k], birds, n, P_Z0, &s);
        if (sets) sets[k] = s;
        if (out) out[k] = d;
    }
    (void)threads;
}

void orc_integrate_all(orc_bird* birds, uint32_t n, int threads) {
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(threads)
#endif
    for (int64_t i = 0; i < (int64_t)n; ++i) orc_step_bird(&birds[i], P_DT);
    (void)threads;
}

/* ---- FP64 twin of one step ------------------------------------------------ */
typedef struct { double x, y, z; } d3;
static inline d3 D(double x, double y, double z) { d3 r = {x, y, z}; return r; }
static inline d3 d_add(d3 a, d3 b) { return D(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline d3 d_sub(d3 a, d3 b) { return D(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline d3 d_mul(d3 a, double s) { return D(a.x * s, a.y * s, a.z * s); }
static inline d3 d_div(d3 a, double s) { return D(a.x / s, a.y / s, a.z / s); }
static inline double d_dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline d3 d_cross(d3 a, d3 b) { return D(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
static inline double d_len(d3 a) { return sqrt(d_dot(a, a)); }
static inline d3 d_normalize(d3 a) { return d_mul(a, 1.0 / d_len(a)); }
static inline double d_clamp(double v, double lo, double hi) { if (v < lo) v = lo; if (v > hi) v = hi; return v; }
static inline d3 d_forward(d3 v) { return d_dot(v, v) > 1e-12 ? d_normalize(v) : D(1, 0, 0); }
static inline d3 d_side(d3 f) { d3 s = d_cross(f, D(0, 0, 1)); return d_dot(s, s) > 1e-8 ? d_normalize(s) : D(1, 0, 0); }
static inline d3 dpos(const orc_bird* b) { return D(b->pos[0], b->pos[1], b->pos[2]); }
static inline d3 dvel(const orc_bird* b) { return D(b->vel[0], b->vel[1], b->vel[2]); }

double orc_step_f64(const orc_bird* birds, uint32_t n, float time_in, double* out, int threads) {
    const double DT = P_DT, DU = P_DU, V0 = P_V0, MASS = P_MASS, G = P_G, L0 = P_L0, D0 = P_D0, TAU = P_TAU;
    const double R_H = P_R_H, SIGMA = P_SIGMA, N_C = P_N_C;
    const double time = (double)(time_in + P_DT); /* the clock itself stays f32, as in the step */
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads)
#endif
    for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
        const uint32_t i = (uint32_t)ii;
        const orc_bird* me = &birds[i];
        d3 steer = D(me->steer[0], me->steer[1], me->steer[2]);
        double radius = me->radius, centrality = me->centrality, next = me->next_decision;
        double neighbours = me->neighbours;
        if (time >= (double)me->next_decision) {
            const d3 p = dpos(me);
            const double r = me->radius;
            const d3 f_i = d_forward(dvel(me));
            d3 sep = D(0, 0, 0), coh = D(0, 0, 0), align = D(0, 0, 0), csum = D(0, 0, 0);
            uint32_t n_all = 0, n_star = 0, n_align = 0, n_g = 0;
            for (uint32_t j = 0; j < n; ++j) {
                if (j == i) continue;
                const d3 d = d_sub(dpos(&birds[j]), p);
                const double d2 = d_dot(d, d);
                if (d2 <= 4.0 * r * r) { csum = d_add(csum, d_div(d, fmax(sqrt(d2), 1e-6))); n_g++; }
                if (d2 > r * r) continue;
                const double dist = sqrt(d2);
                n_all++;
                const d3 dh = d_div(d, fmax(dist, 1e-6));
                const double g = dist <= R_H ? 1.0 : exp(-((dist - R_H) * (dist - R_H)) / (2.0 * SIGMA * SIGMA));
                sep = d_sub(sep, d_mul(dh, g));
                if (dist > R_H) { coh = d_add(coh, dh); n_star++; }
                if (d_dot(f_i, dh) >= (double)P_BLIND_COS) { align = d_add(align, d_forward(dvel(&birds[j]))); n_align++; }
            }
            d3 force = D(0, 0, 0);
            if (n_all) force = d_add(force, d_mul(sep, (double)P_W_SEP / n_all));
            const double cen = n_g ? d_len(csum) / n_g : 0.0;
            if (n_star) { double l = d_len(coh); if (l > 0) force = d_add(force, d_mul(coh, (double)P_W_COH * cen / l)); }
            if (n_align) force = d_add(force, d_mul(d_sub(d_div(align, n_align), f_i), (double)P_W_ALIGN));
            force.z += (double)P_W_ROOST_V * d_clamp(((double)P_Z0 - p.z) / (double)P_H_ROOST_V, -1, 1);
            force = d_add(force, d_mul(f_i, (MASS / TAU) * (V0 - d_len(dvel(me)))));
            steer = force;
            const double nn = n_all > 1 ? n_all : 1;
            radius = d_clamp(r * pow(N_C / nn, (double)P_RADIUS_LERP / 3.0), R_H, (double)P_R_MAX);
            neighbours = n_all;
            centrality = cen;
            next = next + DU;
        }
        /* step_bird in double */
        d3 vel = dvel(me);
        const d3 f = d_forward(vel), side = d_side(f);
        const double speed = fmax(d_len(vel), 1e-6);
        const double a_lat = d_dot(steer, side) / MASS;
        const double maxb = 80.0 * 3.14159265358979323846 / 180.0;
        const double target = d_clamp(atan(a_lat / G), -maxb, maxb);
        const double rate = d_clamp((target - me->roll) / (double)P_TAU_ROLL, -(double)P_MAX_ROLL_RATE, (double)P_MAX_ROLL_RATE);
        const double beta = d_clamp(me->roll + rate * DT, -maxb, maxb);
        const d3 up0 = d_cross(side, f);
        const d3 up = d_add(d_mul(up0, cos(beta)), d_mul(side, sin(beta)));
        const double cb = fmax(cos(beta), 0.2), sr = speed / V0;
        const double lift = sr * sr * L0 / cb, drag = sr * sr * D0;
        d3 flight = d_add(d_sub(d_mul(up, lift), d_mul(f, drag)), d_mul(f, D0));
        flight.z -= MASS * G;
        const d3 control = d_sub(steer, d_mul(side, d_dot(steer, side)));
        vel = d_add(vel, d_mul(d_div(d_add(control, flight), MASS), DT));
        const double sp = d_len(vel);
        if (sp > 2.0 * V0) vel = d_mul(vel, 2.0 * V0 / sp);
        else if (sp < 0.5 * V0 && sp > 1e-6) vel = d_mul(vel, 0.5 * V0 / sp);
        const d3 pos = d_add(dpos(me), d_mul(vel, DT));
        double* w = &out[(size_t)i * 15];
        w[0] = pos.x; w[1] = pos.y; w[2] = pos.z;
        w[3] = vel.x; w[4] = vel.y; w[5] = vel.z;
        w[6] = beta; w[7] = rate; w[8] = radius;
        w[9] = steer.x; w[10] = steer.y; w[11] = steer.z;
        w[12] = next; w[13] = neighbours; w[14] = centrality;
    }
    (void)threads;
    return time;
}

/* ---- grid: cuda/flock.cu:75-83, 368-372 ----------------------------------- */
uint32_t orc_buckets_for(uint32_t n) {
    uint64_t want = 1;
    while (want < (uint64_t)n * 2) want <<= 1;
    if (want < (1u << 16)) want = 1u << 16;
    if (want > (1u << 22)) want = 1u << 22;
    return (uint32_t)want;
}

void orc_cell_of(const float p[3], int32_t c[3]) {
    const float inv = 1.0f / P_GRID_CELL;
    for (int k = 0; k < 3; ++k) c[k] = (int32_t)floorf(p[k] * inv);
}

uint32_t orc_bucket_of(const int32_t c[3], uint32_t mask) {
    uint32_t h = ((uint32_t)c[0] * 73856093u) ^ ((uint32_t)c[1] * 19349663u) ^ ((uint32_t)c[2] * 83492791u);
    return h & mask;
}

void orc_grid(const orc_bird* birds, uint32_t n, uint32_t buckets, uint32_t* keys, uint32_t* offsets, uint32_t* sorted) {
    uint32_t* cursor = (uint32_t*)calloc(buckets, sizeof(uint32_t));
    for (uint32_t i = 0; i < n; ++i) {
        int32_t c[3];
        orc_cell_of(birds[i].pos, c);
        keys[i] = orc_bucket_of(c, buckets - 1u);
        cursor[keys[i]]++;
    }
    uint32_t run = 0;
    for (uint32_t b = 0; b < buckets; ++b) {
        offsets[b] = run;
        run += cursor[b];
        cursor[b] = offsets[b];
    }
    offsets[buckets] = run;
    for (uint32_t i = 0; i < n; ++i) sorted[cursor[keys[i]]++] = i;
    free(cursor);
}

int orc_check_grid(const uint32_t* keys, const uint32_t* offsets, const uint32_t* sorted, uint32_t n, uint32_t buckets,
                   const orc_bird* birds) {
    for (uint32_t i = 0; i < n; ++i)
        if (keys[i] >= buckets) return 1; /* bucket index outside 0..buckets (hash/count) */
    if (offsets[0] != 0) return 2;        /* scan start */
    if (offsets[buckets] != n) return 3;  /* scan total */
    for (uint32_t b = 0; b < buckets; ++b)
        if (offsets[b + 1] < offsets[b]) return 4; /* offsets decrease */
    uint32_t* count = (uint32_t*)calloc(buckets, sizeof(uint32_t));
    uint8_t* seen = (uint8_t*)calloc(n ? n : 1, 1);
    int rc = 0;
    for (uint32_t i = 0; i < n; ++i) count[keys[i]]++;
    for (uint32_t b = 0; b < buckets && !rc; ++b)
        if (offsets[b + 1] - offsets[b] != count[b]) rc = 5; /* range size vs count */
    for (uint32_t b = 0; b < buckets && !rc; ++b) {
        for (uint32_t s = offsets[b]; s < offsets[b + 1] && !rc; ++s) {
            uint32_t j = sorted[s];
            if (j >= n || seen[j]) { rc = 6; break; } /* not a permutation */
            seen[j] = 1;
            if (keys[j] != b) { rc = 7; break; }      /* bird in a foreign range */
            if (s > offsets[b] && sorted[s - 1] >= j) { rc = 8; break; } /* not stable (bird order) */
        }
    }
    if (!rc && birds) {
        for (uint32_t i = 0; i < n && !rc; ++i) {
            int32_t c[3];
            orc_cell_of(birds[i].pos, c);
            if (orc_bucket_of(c, buckets - 1u) != keys[i]) rc = 9; /* key is not the cell hash */
        }
    }
    free(count);
    free(seen);
    return rc;
}

/* ---- main.rs:83-208 ------------------------------------------------------- */
void orc_stats(const orc_bird* b, uint32_t n, float out[4]) {
    const float nf = (float)n;
    float speed = 0.0f, nb = 0.0f, radius = 0.0f;
    v3 pol = V0V;
    for (uint32_t i = 0; i < n; ++i) speed += v_len(vel_of(&b[i]));
    for (uint32_t i = 0; i < n; ++i) nb += (float)b[i].neighbours;
    for (uint32_t i = 0; i < n; ++i) radius += b[i].radius;
    for (uint32_t i = 0; i < n; ++i) pol = v_add(pol, forward(vel_of(&b[i])));
    out[0] = speed / nf;
    out[1] = nb / nf;
    out[2] = radius / nf;
    out[3] = v_len(v_div(pol, nf));
}

int orc_statdiff(const orc_bird* a, const orc_bird* b, uint32_t n, float out[4]) {
    float sa[4], sb[4];
    const float tol[4] = {0.02f, 0.1f, 0.01f, 0.005f};
    orc_stats(a, n, sa);
    orc_stats(b, n, sb);
    int ok = 1;
    for (int k = 0; k < 4; ++k) {
        out[k] = fabsf(sa[k] - sb[k]);
        ok &= out[k] <= tol[k];
    }
    return ok;
}

static inline float absmax3(const float* x, const float* y) {
    float m = fabsf(x[0] - y[0]);
    float t = fabsf(x[1] - y[1]);
    if (t > m) m = t;
    t = fabsf(x[2] - y[2]);
    if (t > m) m = t;
    return m;
}

int orc_diff(const orc_bird* a, const orc_bird* b, uint32_t n, float pos_tol, float vel_tol, uint32_t allow,
             float outlier_max, float out[7], uint32_t* mismatch, uint32_t* outliers) {
    float dp = 0, dv = 0, dr = 0, dc = 0, ds = 0, droll = 0, dspin = 0;
    uint32_t nout = 0, nbm = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const orc_bird* x = &a[i];
        const orc_bird* y = &b[i];
        float bp = absmax3(x->pos, y->pos), bv = absmax3(x->vel, y->vel);
        dp = fmaxf(dp, bp);
        dv = fmaxf(dv, bv);
        nout += (bp > pos_tol || bv > vel_tol);
        dr = fmaxf(dr, fabsf(x->radius - y->radius));
        dc = fmaxf(dc, fabsf(x->centrality - y->centrality));
        ds = fmaxf(ds, absmax3(x->steer, y->steer));
        droll = fmaxf(droll, fabsf(x->roll - y->roll));
        dspin = fmaxf(dspin, fabsf(x->spin - y->spin));
        nbm += x->neighbours != y->neighbours;
    }
    out[0] = dp; out[1] = dv; out[2] = dr; out[3] = dc; out[4] = ds; out[5] = droll; out[6] = dspin;
    *mismatch = nbm;
    *outliers = nout;
    if (allow == 0) return dp <= pos_tol && dv <= vel_tol && nbm == 0;
    return nout <= allow && dp <= outlier_max && dv <= outlier_max && nbm == 0;
}

/* ---- CPU grid step: the reference GPU backend's algorithm on host cores ----
 * cuda/flock.cu:190-290 (decide) restated for the CPU: per deciding bird, an
 * R walk over the cells of [cell(p - r), cell(p + r)] that pass the sphere
 * test with its +1e-4 slack (flock.cu:85-91), each cell's bucket range with
 * the exact cell check (flock.cu:219-221), then the same walk for 2R
 * (centrality). The grid is the stable counting sort above. OpenMP over the
 * deciding birds and over integrate. Used only as a timed CPU baseline and
 * checked against orc_step in the tests. */
static int cell_hits_sphere(const int32_t c[3], v3 p, float r2) {
    const float lx = (float)c[0] * P_GRID_CELL, ly = (float)c[1] * P_GRID_CELL, lz = (float)c[2] * P_GRID_CELL;
    const float dx = f_clamp(p.x, lx, lx + P_GRID_CELL) - p.x;
    const float dy = f_clamp(p.y, ly, ly + P_GRID_CELL) - p.y;
    const float dz = f_clamp(p.z, lz, lz + P_GRID_CELL) - p.z;
    return dx * dx + dy * dy + dz * dz <= r2 + 1e-4f;
}

static orc_decision grid_decide(uint32_t i, const orc_bird* birds, const uint32_t* offsets, const uint32_t* sorted,
                                uint32_t mask) {
    const orc_bird* me = &birds[i];
    const v3 p = pos_of(me);
    const float r = me->radius;
    const v3 f_i = forward(vel_of(me));
    v3 sep = V0V, coh = V0V, align = V0V, csum = V0V;
    uint32_t n_all = 0, n_star = 0, n_align = 0, n_g = 0;
    for (int walk = 0; walk < 2; ++walk) {
        const float rr = walk == 0 ? r : 2.0f * r;
        const float r2 = walk == 0 ? r * r : 4.0f * r * r;
        const float lo_p[3] = {p.x - rr, p.y - rr, p.z - rr}, hi_p[3] = {p.x + rr, p.y + rr, p.z + rr};
        int32_t lo[3], hi[3], c[3], cq[3];
        orc_cell_of(lo_p, lo);
        orc_cell_of(hi_p, hi);
        for (c[2] = lo[2]; c[2] <= hi[2]; ++c[2])
            for (c[1] = lo[1]; c[1] <= hi[1]; ++c[1])
                for (c[0] = lo[0]; c[0] <= hi[0]; ++c[0]) {
                    if (!cell_hits_sphere(c, p, r2)) continue;
                    const uint32_t b = orc_bucket_of(c, mask);
                    for (uint32_t s = offsets[b]; s < offsets[b + 1]; ++s) {
                        const uint32_t j = sorted[s];
                        if (j == i) continue;
                        orc_cell_of(birds[j].pos, cq);
                        if (cq[0] != c[0] || cq[1] != c[1] || cq[2] != c[2]) continue;
                        const v3 d = v_sub(pos_of(&birds[j]), p);
                        const float d2 = v_dot(d, d);
                        if (d2 > r2) continue;
                        const float dist = sqrtf(d2);
                        const v3 dhat = v_div(d, f_max(dist, 1e-6f));
                        if (walk == 1) {
                            csum = v_add(csum, dhat);
                            n_g += 1;
                            continue;
                        }
                        n_all += 1;
                        float g = 1.0f;
                        if (dist > P_R_H) {
                            const float t = dist - P_R_H;
                            g = expf(-(t * t) / (2.0f * P_SIGMA * P_SIGMA));
                        }
                        sep = v_sub(sep, v_mul(dhat, g));
                        if (dist > P_R_H) {
                            coh = v_add(coh, dhat);
                            n_star += 1;
                        }
                        if (v_dot(f_i, dhat) >= P_BLIND_COS) {
                            align = v_add(align, forward(vel_of(&birds[j])));
                            n_align += 1;
                        }
                    }
                }
    }
    v3 force = V0V;
    if (n_all > 0) force = v_add(force, v_mul(sep, P_W_SEP / (float)n_all));
    const float centrality = n_g > 0 ? v_len(csum) / (float)n_g : 0.0f;
    if (n_star > 0) force = v_add(force, v_mul(v_normalize_or_zero(coh), P_W_COH * centrality));
    const v3 a = n_align > 0 ? v_sub(v_div(align, (float)n_align), f_i) : V0V;
    force = v_add(force, v_mul(a, P_W_ALIGN));
    force = v_add(force, v_mul(VZ, P_W_ROOST_V * f_clamp((P_Z0 - p.z) / P_H_ROOST_V, -1.0f, 1.0f)));
    const float speed = v_len(vel_of(me));
    force = v_add(force, v_mul(f_i, (P_MASS / P_TAU) * (P_V0 - speed)));
    orc_decision out;
    out.force[0] = force.x; out.force[1] = force.y; out.force[2] = force.z;
    out.radius = orc_radius_step(r, n_all);
    out.neighbours = n_all;
    out.centrality = centrality;
    return out;
}

float orc_step_grid(orc_bird* birds, uint32_t n, float time, int threads) {
    time += P_DT;
    const uint32_t buckets = orc_buckets_for(n);
    uint32_t* keys = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint32_t* offsets = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)buckets + 1));
    uint32_t* sorted = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    orc_decision* dec = (orc_decision*)malloc(sizeof(orc_decision) * (n ? n : 1));
    orc_grid(birds, n, buckets, keys, offsets, sorted);
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
#endif
    for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
        const uint32_t i = (uint32_t)ii;
        if (time >= birds[i].next_decision) dec[i] = grid_decide(i, birds, offsets, sorted, buckets - 1u);
    }
    for (uint32_t i = 0; i < n; ++i) {
        if (!(time >= birds[i].next_decision)) continue;
        birds[i].steer[0] = dec[i].force[0];
        birds[i].steer[1] = dec[i].force[1];
        birds[i].steer[2] = dec[i].force[2];
        birds[i].radius = dec[i].radius;
        birds[i].neighbours = dec[i].neighbours;
        birds[i].centrality = dec[i].centrality;
        birds[i].next_decision += P_DU;
    }
    orc_integrate_all(birds, n, threads);
    free(keys);
    free(offsets);
    free(sorted);
    free(dec);
    (void)threads;
    return time;
}
