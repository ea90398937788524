// Pass 5: decide (reference crates/flock-ref/src/model.rs:53-145; cuda/flock.cu:190-290),
// one warp per deciding bird.
//
// The warp first builds the bird's 2R neighbourhood: the cells of a
// conservative box that intersect the (inflated) 2R sphere. With at most 32
// cells (2R < 4 m, the usual case), each lane takes one cell and duplicate
// buckets are dropped with __match_any_sync, so every bucket is swept once and
// needs no per-candidate cell check. Wider boxes walk the cells 32 at a time
// with the reference's exact cell check (cuda/flock.cu:219-221), and a box
// wider than the flock itself sweeps the flock's whole range.
//
// Each bucket's birds are contiguous in the cell-ordered float4 view, so the
// lanes of a warp read one coalesced 512 B run per cell. The sweep is split in
// two: the cheap phase computes d2 for every candidate and appends the indices
// of those within 2R to a per-warp queue in shared memory (ballot + popc);
// whenever 32 hits are queued, the whole warp processes them together in the
// expensive phase (sqrt, three IEEE divisions, the separation Gaussian,
// blind-angle test). Only ~11 % of candidates are hits, so this keeps the
// expensive code on full warps instead of running it for one or two lanes.
//
// Per-lane partial sums are reduced with a fixed shuffle pattern; lane 0
// finishes the decision in the oracle's order of operations.
#pragma once

#include "device_common.cuh"

namespace flk {

struct Acc {
    f3 sep, coh, align, csum;
    uint32_t n_all, n_star, n_align, n_g;
    uint32_t h_all, h_star, h_align, h_g;
};

__device__ __forceinline__ uint32_t set_mix(uint32_t j) {
    uint32_t h = j + 1u;
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

// Bucket range [s, e) of bucket b; an inconsistent range (only possible if the
// scan gave up) is recorded and treated as empty instead of being read.
__device__ __forceinline__ void bucket_range(const uint32_t* __restrict__ offsets, uint32_t b, uint32_t V,
                                             StepCtl* __restrict__ ctl, uint32_t& s, uint32_t& e) {
    s = __ldg(&offsets[b]);
    e = __ldg(&offsets[b + 1]);
    if (e < s || e > V) {
        atomicCAS(&ctl->error, 0u, (uint32_t)DEV_BAD_RANGE);
        e = s = 0;
    }
}

// Everything a lane needs while sweeping one deciding bird's neighbourhood.
struct Sweep {
    f3 p, fi;
    float r2, c2;
    uint32_t self;
    const float4* __restrict__ spos;
    const float4* __restrict__ sfwd;
    uint32_t* q;  // this warp's 64-entry hit queue (shared memory)
    uint32_t qn;  // entries queued (warp-uniform)
    Acc a;
};

// Expensive phase for one hit t (d2 <= c2 already established).
template <bool SETS>
__device__ __forceinline__ void take(Sweep& w, uint32_t t) {
    const float4 q = __ldg(&w.spos[t]);
    const f3 d = mk(__fsub_rn(q.x, w.p.x), __fsub_rn(q.y, w.p.y), __fsub_rn(q.z, w.p.z));
    const float d2 = dot(d, d);
    const float dist = __fsqrt_rn(d2);
    const f3 dh = dvs(d, fmaxf(dist, 1e-6f));
    w.a.csum = add(w.a.csum, dh);
    w.a.n_g += 1;
    const uint32_t j = __float_as_uint(q.w);
    if (SETS) w.a.h_g += set_mix(j);
    if (d2 > w.r2) return;
    w.a.n_all += 1;
    if (SETS) w.a.h_all += set_mix(j);
    float g = 1.0f;
    if (dist > R_H) {
        const float tt = __fsub_rn(dist, R_H);
        g = expf(__fdiv_rn(-__fmul_rn(tt, tt), TWO_SIGMA2));
    }
    w.a.sep = sub(w.a.sep, mul(dh, g));
    if (dist > R_H) {
        w.a.coh = add(w.a.coh, dh);
        w.a.n_star += 1;
        if (SETS) w.a.h_star += set_mix(j);
    }
    if (dot(w.fi, dh) >= BLIND_COS) {
        const float4 fw = __ldg(&w.sfwd[t]);
        w.a.align = add(w.a.align, xyz(fw));
        w.a.n_align += 1;
        if (SETS) w.a.h_align += set_mix(j);
    }
}

// Cheap phase over the contiguous candidate range [sc, ec). CHECK_CELL: only
// birds of cell (cx, cy, cz) count (cell walk, where a bucket can repeat).
template <bool SETS, bool CHECK_CELL>
__device__ __forceinline__ void sweep(Sweep& w, uint32_t sc, uint32_t ec, uint32_t lane, int cx = 0, int cy = 0,
                                      int cz = 0) {
    for (uint32_t base = sc; base < ec; base += 32) {
        const uint32_t t = base + lane;
        bool hit = false;
        if (t < ec && t != w.self) {
            const float4 q = __ldg(&w.spos[t]);
            const float dx = __fsub_rn(q.x, w.p.x), dy = __fsub_rn(q.y, w.p.y), dz = __fsub_rn(q.z, w.p.z);
            const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            hit = d2 <= w.c2;
            if (CHECK_CELL) hit = hit && cell1(q.x) == cx && cell1(q.y) == cy && cell1(q.z) == cz;
        }
        const uint32_t hm = __ballot_sync(FULL, hit);
        if (hm) {
            if (hit) w.q[w.qn + __popc(hm & lanemask_lt())] = t;
            w.qn += __popc(hm);
            if (w.qn >= 32) {
                __syncwarp();
                take<SETS>(w, w.q[lane]);
                const uint32_t extra = w.qn - 32;
                const uint32_t moved = lane < extra ? w.q[32 + lane] : 0u;
                __syncwarp();
                if (lane < extra) w.q[lane] = moved;
                __syncwarp();
                w.qn = extra;
            }
        }
    }
}

template <bool SETS>
__device__ __forceinline__ void drain(Sweep& w, uint32_t lane) {
    if (w.qn) {
        __syncwarp();
        if (lane < w.qn) take<SETS>(w, w.q[lane]);
        __syncwarp();
        w.qn = 0;
    }
}

__device__ __forceinline__ float wsum(float x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = __fadd_rn(x, __shfl_xor_sync(FULL, x, o));
    return x;
}
__device__ __forceinline__ uint32_t wsumu(uint32_t x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
    return x;
}
__device__ __forceinline__ f3 wsum3(f3 v) { return mk(wsum(v.x), wsum(v.y), wsum(v.z)); }

// params.rs:61-65 with the tabulated factor
__device__ __forceinline__ float radius_step(float r, uint32_t n, const float* __restrict__ rtab) {
    const float factor = n < (uint32_t)RADIUS_TABLE ? __ldg(&rtab[n]) : powf(__fdiv_rn(N_C, (float)n), RADIUS_EXP);
    return clampf(__fmul_rn(r, factor), R_H, R_MAX);
}

// CTAs of 256 threads the register budget is sized for (4 -> 64 registers).
#ifndef FLK_DECIDE_MIN_BLOCKS
#define FLK_DECIDE_MIN_BLOCKS 4
#endif

// Shared memory: 64 queue entries (256 B) per warp.
template <bool SETS>
__global__ void __launch_bounds__(256, FLK_DECIDE_MIN_BLOCKS) k_decide(const FlockDesc* __restrict__ fl, uint32_t V,
                                                   StepCtl* __restrict__ ctl, const uint2* __restrict__ due,
                                                   const uint32_t* __restrict__ offsets,
                                                   const float4* __restrict__ spos, const float4* __restrict__ sfwd,
                                                   const float4* __restrict__ Bv, float4* __restrict__ C,
                                                   float4* __restrict__ D, const float* __restrict__ rtab,
                                                   uint32_t* __restrict__ sets) {
    extern __shared__ uint32_t s_queue[];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t ndue = *(volatile uint32_t*)&ctl->due_count;
    uint32_t cand = 0, pairs = 0;  // per-warp totals (fit easily in 32 bits)

    Sweep w;
    w.spos = spos;
    w.sfwd = sfwd;
    w.q = s_queue + (threadIdx.x >> 5) * 64;
    w.qn = 0;

    for (uint32_t e = gw; e < ndue; e += nw) {
        const uint2 ent = due[e];
        const uint32_t k = ent.x;
        const FlockDesc d = fl[ent.y];
        const float4 me = spos[k];
        const uint32_t local = __float_as_uint(me.w);
        const uint32_t st = d.sbase + local;
        const float r = C[st].w;
        w.p = mk(me.x, me.y, me.z);
        w.fi = forward(xyz(Bv[st]));
        w.r2 = __fmul_rn(r, r);
        const float rr = __fmul_rn(2.0f, r);
        w.c2 = __fmul_rn(rr, rr);
        w.self = k;
        const f3 p = w.p;
        // Search reach: 2r inflated so every bird the exact test d2 <= c2 accepts
        // lies in a visited cell (covers the rounding of p -/+ reach as well).
        const float pm = fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z)));
        const float reach = rr * 1.00001f + 1e-3f + pm * 1e-6f;
        const float reach2 = reach * reach;
        const int lx = cell1(p.x - reach), ly = cell1(p.y - reach), lz = cell1(p.z - reach);
        const long long nxl = (long long)cell1(p.x + reach) - lx + 1, nyl = (long long)cell1(p.y + reach) - ly + 1,
                        nzl = (long long)cell1(p.z + reach) - lz + 1;
        // an absurd reach (huge or non-finite radius) takes the brute-force path below
        const bool wide = nxl > (1 << 20) || nyl > (1 << 20) || nzl > (1 << 20);
        const long long ncell = wide ? (1ll << 62) : nxl * nyl * nzl;
        const int nx = (int)nxl, ny = (int)nyl;
        const uint32_t mask = d.buckets - 1u;

        w.a.sep = w.a.coh = w.a.align = w.a.csum = mk(0.f, 0.f, 0.f);
        w.a.n_all = w.a.n_star = w.a.n_align = w.a.n_g = 0;
        w.a.h_all = w.a.h_star = w.a.h_align = w.a.h_g = 0;

        if (ncell <= 32) {
            // fast path: each distinct bucket of the culled box once, no cell check
            bool valid = false;
            uint32_t b = 0;
            if ((long long)lane < ncell) {
                const int cx = lx + (int)lane % nx;
                const int t = (int)lane / nx;
                const int cy = ly + t % ny, cz = lz + t / ny;
                const float ox = (float)cx * GRID_CELL, oy = (float)cy * GRID_CELL, oz = (float)cz * GRID_CELL;
                const float dx = fminf(fmaxf(p.x, ox), ox + GRID_CELL) - p.x;
                const float dy = fminf(fmaxf(p.y, oy), oy + GRID_CELL) - p.y;
                const float dz = fminf(fmaxf(p.z, oz), oz + GRID_CELL) - p.z;
                valid = dx * dx + dy * dy + dz * dz <= reach2;
                b = d.bbase + (cell_hash(cx, cy, cz) & mask);
            }
            const uint32_t vm = __ballot_sync(FULL, valid);
            bool keep = false;
            if (valid) {
                const uint32_t peers = __match_any_sync(vm, b);
                keep = (int)lane == __ffs(peers) - 1;
            }
            uint32_t s = 0, en = 0;
            if (keep) bucket_range(offsets, b, V, ctl, s, en);
            uint32_t km = __ballot_sync(FULL, en > s);
            while (km) {
                const int c = __ffs(km) - 1;
                km &= km - 1;
                const uint32_t sc = __shfl_sync(FULL, s, c), ec = __shfl_sync(FULL, en, c);
                cand += ec - sc;
                sweep<SETS, false>(w, sc, ec, lane);
            }
        } else {
            uint32_t f0 = __ldg(&offsets[d.bbase]), f1 = __ldg(&offsets[d.bbase + d.buckets]);
            if (f1 < f0 || f1 > V) f1 = f0 = 0;
            if (ncell * 16 >= (long long)(f1 - f0)) {
                // very wide reach: brute force over the flock's own range
                cand += f1 - f0;
                sweep<SETS, false>(w, f0, f1, lane);
            } else {
                // cell walk with the exact cell check (buckets may repeat)
                for (long long c0 = 0; c0 < ncell; c0 += 32) {
                    const long long ci = c0 + lane;
                    bool valid = false;
                    int cx = 0, cy = 0, cz = 0;
                    uint32_t s = 0, en = 0;
                    if (ci < ncell) {
                        cx = lx + (int)(ci % nxl);
                        const long long t = ci / nxl;
                        cy = ly + (int)(t % nyl);
                        cz = lz + (int)(t / nyl);
                        const float ox = (float)cx * GRID_CELL, oy = (float)cy * GRID_CELL, oz = (float)cz * GRID_CELL;
                        const float dx = fminf(fmaxf(p.x, ox), ox + GRID_CELL) - p.x;
                        const float dy = fminf(fmaxf(p.y, oy), oy + GRID_CELL) - p.y;
                        const float dz = fminf(fmaxf(p.z, oz), oz + GRID_CELL) - p.z;
                        valid = dx * dx + dy * dy + dz * dz <= reach2;
                        if (valid) {
                            bucket_range(offsets, d.bbase + (cell_hash(cx, cy, cz) & mask), V, ctl, s, en);
                            valid = en > s;
                        }
                    }
                    uint32_t km = __ballot_sync(FULL, valid);
                    while (km) {
                        const int c = __ffs(km) - 1;
                        km &= km - 1;
                        const uint32_t sc = __shfl_sync(FULL, s, c), ec = __shfl_sync(FULL, en, c);
                        const int ccx = __shfl_sync(FULL, cx, c), ccy = __shfl_sync(FULL, cy, c),
                                  ccz = __shfl_sync(FULL, cz, c);
                        cand += ec - sc;
                        sweep<SETS, true>(w, sc, ec, lane, ccx, ccy, ccz);
                    }
                }
            }
        }
        drain<SETS>(w, lane);

        // warp reduction (fixed butterfly; lane 0's association is deterministic)
        const f3 sep = wsum3(w.a.sep), coh = wsum3(w.a.coh), align = wsum3(w.a.align), csum = wsum3(w.a.csum);
        const uint32_t n_all = wsumu(w.a.n_all), n_star = wsumu(w.a.n_star), n_align = wsumu(w.a.n_align),
                       n_g = wsumu(w.a.n_g);
        uint32_t h_all = 0, h_star = 0, h_align = 0, h_g = 0;
        if (SETS) {
            h_all = wsumu(w.a.h_all);
            h_star = wsumu(w.a.h_star);
            h_align = wsumu(w.a.h_align);
            h_g = wsumu(w.a.h_g);
        }
        if (lane == 0) {
            pairs += n_g;
            f3 force = mk(0.f, 0.f, 0.f);
            if (n_all > 0) force = add(force, mul(sep, __fdiv_rn(W_SEP, (float)n_all)));
            const float cen = n_g > 0 ? __fdiv_rn(len(csum), (float)n_g) : 0.0f;
            if (n_star > 0) force = add(force, mul(normalize_or_zero(coh), __fmul_rn(W_COH, cen)));
            const f3 al = n_align > 0 ? sub(dvs(align, (float)n_align), w.fi) : mk(0.f, 0.f, 0.f);
            force = add(force, mul(al, W_ALIGN));
            const float roost = __fmul_rn(W_ROOST_V, clampf(__fdiv_rn(__fsub_rn(Z0, p.z), H_ROOST_V), -1.0f, 1.0f));
            force = add(force, mul(mk(0.f, 0.f, 1.f), roost));
            const float speed = len(xyz(Bv[st]));  // reloaded: not kept live across the sweep
            force = add(force, mul(w.fi, __fmul_rn(MASS / TAU, __fsub_rn(V0, speed))));
            const float nd = D[st].x;
            C[st] = make_float4(force.x, force.y, force.z, radius_step(C[st].w, n_all, rtab));
            D[st] = make_float4(__fadd_rn(nd, DU), __uint_as_float(n_all), cen, 0.f);
            if (SETS) {
                uint32_t* o = sets + (size_t)(d.vbase + local) * 8;
                o[0] = n_all; o[1] = n_star; o[2] = n_align; o[3] = n_g;
                o[4] = h_all; o[5] = h_star; o[6] = h_align; o[7] = h_g;
            }
        }
    }
    // per-warp totals straight to the counters (no block barrier)
    if (lane == 0) {
        if (cand) atomicAdd(&ctl->cand_total, (unsigned long long)cand);
        if (pairs) atomicAdd(&ctl->pair_total, (unsigned long long)pairs);
        if (gw == 0) atomicAdd(&ctl->due_total, (unsigned long long)ndue);
    }
}

}  // namespace flk
