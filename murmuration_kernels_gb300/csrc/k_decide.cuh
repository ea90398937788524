// Pass 5: decide (reference crates/flock-ref/src/model.rs:53-145; cuda/flock.cu:190-290),
// one warp per deciding bird.
//
// The warp first builds the bird's 2R neighbourhood: the cells of a
// conservative box that intersect the (inflated) 2R sphere. With at most 32
// cells (2R below about one cell edge, the usual case), each lane takes one cell; every bucket is
// swept once and needs no per-candidate cell check (grid-reporting steps drop
// the reference hash's duplicate buckets with __match_any_sync; the production
// lattice index never repeats within such a box). Wider boxes walk the cells 32 at a time
// with the reference's exact cell check (cuda/flock.cu:219-221), and a box
// wider than the flock itself sweeps the flock's whole range.
//
// Each bucket's birds are contiguous in the flock's state, which the sort
// pass has just written in cell order (view index t lives in slot t + shift of
// the reordered buffer), so the lanes of a warp read coalesced runs of
// positions. In production steps each run is ordered by 1 m z-slab and the
// sort recorded the slab boundaries, so every visited cell's run is narrowed
// to the slabs the bird's z-reach touches. The sweep is split in two: the
// cheap phase computes d2 for every candidate and appends the indices of those
// within 2R to a per-warp queue in shared memory (ballot + popc); whenever 32
// hits are queued, the whole warp processes them together in the expensive
// phase (sqrt, three IEEE divisions, the separation Gaussian, blind-angle
// test). Only ~19 % of candidates are hits, so this keeps the expensive code on
// full warps instead of running it for a few lanes. The cheap phase sweeps the
// bucket ranges as one packed sequence, two 32-candidate chunks per iteration
// (two loads in flight per lane).
// The per-bird box arithmetic runs one bird per lane for a warp's next
// DECIDE_BATCH birds (group_boxes), not warp-uniformly.
//
// Per-lane partial sums are reduced with a transposed (reduce-scatter)
// shuffle pattern straight into shared memory; once DECIDE_BATCH birds are
// reduced, the lanes finish their decisions at once, one bird per lane, in the
// oracle's order of operations.
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

// Bucket range [s, e) of bucket b: its start (offsets) and length (counts). An
// empty bucket's start is stale and never used; an inconsistent range (only
// possible if the grid build gave up) is recorded and treated as empty. The
// range's slots [s + shift, e + shift) must also lie inside the state arrays
// (lim = 2 * cap entries).
__device__ __forceinline__ void bucket_range(const uint32_t* __restrict__ offsets,
                                             const uint32_t* __restrict__ counts, uint32_t b, uint32_t V,
                                             uint32_t shift, uint32_t lim, StepCtl* __restrict__ ctl, uint32_t& s,
                                             uint32_t& e) {
    const uint32_t c = __ldg(&counts[b]);
    s = __ldg(&offsets[b]);
    e = s + c;
    const uint32_t ss = s + shift;
    if (c == 0) {
        e = s = 0;
    } else if (e < s || e > V || ss + c < ss || ss + c > lim) {
        atomicCAS(&ctl->error, 0u, (uint32_t)DEV_BAD_RANGE);
        e = s = 0;
    }
}

// Everything a lane needs while sweeping one deciding bird's neighbourhood.
struct Sweep {
    f3 p, fi;
    float r2, c2;
    uint32_t self;
    uint32_t shift;                   // slot - view index of the bird's flock
    const float4* __restrict__ pos;   // state: position, roll (by slot)
    const uint32_t* __restrict__ bid;  // state: bird index (by slot)
    const float4* __restrict__ sfwd;  // unit headings (by view index)
    uint32_t* q;  // this warp's 96-entry hit queue (shared memory)
    uint32_t qn;  // entries queued (warp-uniform)
    Acc a;
};

// A candidate's position: from the state through the read-only cache, or
// (STG) from positions the CTA staged in shared memory.
template <bool STG>
__device__ __forceinline__ float4 ldpos(const float4* p) {
    if (STG) return *p;
    return __ldg(p);
}

// Expensive phase for one hit t: a member of the R set in production steps
// (the sweep summed its 2R share, ring), of the 2R set in grid-reporting
// steps (d2 <= c2 already established). STG: t is an index into the staged
// positions, whose .w holds the candidate's view index.
template <bool SETS, bool STG = false>
__device__ __forceinline__ void take(Sweep& w, uint32_t t) {
    const float4 q = ldpos<STG>(&w.pos[t + w.shift]);
    // the neighbour's heading is needed only inside the blind cone, but
    // loading it here, before the arithmetic, hides the load's latency
    const float4 fw = __ldg(&w.sfwd[STG ? __float_as_uint(q.w) : t]);
    const f3 d = mk(__fsub_rn(q.x, w.p.x), __fsub_rn(q.y, w.p.y), __fsub_rn(q.z, w.p.z));
    const float d2 = dot(d, d);
    const float dist = __fsqrt_rn(d2);
    const f3 dh = dvs(d, fmaxf(dist, 1e-6f));
    const uint32_t j = SETS ? __ldg(&w.bid[t + w.shift]) : 0u;
    if (SETS) {  // production steps add the 2R set's share in the sweep (ring) and queue only hits inside R
        w.a.csum = add(w.a.csum, dh);
        w.a.n_g += 1;
        w.a.h_g += set_mix(j);
        if (d2 > w.r2) return;
    }
    w.a.n_all += 1;
    if (SETS) w.a.h_all += set_mix(j);
    // the separation Gaussian only weights a sum (compared to rounding), so it
    // takes the fast exponential and a multiplication by 1 / (2 sigma^2)
    float g = 1.0f;
    if (dist > R_H) {
        const float tt = __fsub_rn(dist, R_H);
        g = __expf(__fmul_rn(-__fmul_rn(tt, tt), 1.0f / TWO_SIGMA2));
    }
    w.a.sep = sub(w.a.sep, mul(dh, g));
    if (dist > R_H) {
        w.a.coh = add(w.a.coh, dh);
        w.a.n_star += 1;
        if (SETS) w.a.h_star += set_mix(j);
    }
    if (dot(w.fi, dh) >= BLIND_COS) {
        w.a.align = add(w.a.align, xyz(fw));
        w.a.n_align += 1;
        if (SETS) w.a.h_align += set_mix(j);
    }
}

// Queues the lanes' hits; when 32 are waiting, the whole warp takes them.
template <bool SETS, bool STG = false>
__device__ __forceinline__ void enqueue(Sweep& w, bool hit, uint32_t t, uint32_t lane) {
    const uint32_t hm = __ballot_sync(FULL, hit);
    if (!hm) return;
    if (hit) w.q[w.qn + __popc(hm & lanemask_lt())] = t;
    w.qn += __popc(hm);
    if (w.qn >= 32) {
        __syncwarp();
        take<SETS, STG>(w, w.q[lane]);
        const uint32_t extra = w.qn - 32;
        const uint32_t moved = lane < extra ? w.q[32 + lane] : 0u;
        __syncwarp();
        if (lane < extra) w.q[lane] = moved;
        __syncwarp();
        w.qn = extra;
    }
}

// Queues two chunks' hits at once (A's, then B's, the order of two single
// enqueues) and takes full batches of 32. Hit k of the bird still goes to lane
// k mod 32, so the sums are the same as with one chunk per enqueue.
template <bool SETS, bool STG = false>
__device__ __forceinline__ void enqueue2(Sweep& w, bool hA, uint32_t tA, bool hB, uint32_t tB, uint32_t lane) {
    const uint32_t ma = __ballot_sync(FULL, hA), mb = __ballot_sync(FULL, hB);
    if (!(ma | mb)) return;
    const uint32_t lt = lanemask_lt(), na = __popc(ma);
    if (hA) w.q[w.qn + __popc(ma & lt)] = tA;
    if (hB) w.q[w.qn + na + __popc(mb & lt)] = tB;
    w.qn += na + __popc(mb);
    while (w.qn >= 32) {
        __syncwarp();
        take<SETS, STG>(w, w.q[lane]);
        const uint32_t extra = w.qn - 32;
        const uint32_t m0 = lane < extra ? w.q[32 + lane] : 0u;
        const uint32_t m1 = lane + 32 < extra ? w.q[64 + lane] : 0u;
        __syncwarp();
        if (lane < extra) w.q[lane] = m0;
        if (lane + 32 < extra) w.q[32 + lane] = m1;
        __syncwarp();
        w.qn = extra;
    }
}

// Offset d from the deciding bird to candidate position q, and |d|^2. Set
// membership must round exactly as the oracle's chain of separately rounded
// f32 operations, so the test stays in scalar round-to-nearest intrinsics:
// paired f32x2 multiplies and adds (the __fmul2_rn/__fadd2_rn intrinsics, or
// mul.rn/add.rn.f32x2 in PTX) were measured to round d2 differently, admitting
// a bird one ulp outside 2R (test_two_birds_one_ulp_outside_2r), and cost no
// time to give up.
__device__ __forceinline__ float offset2(const Sweep& w, const float4 q, f3& d) {
    d = mk(__fsub_rn(q.x, w.p.x), __fsub_rn(q.y, w.p.y), __fsub_rn(q.z, w.p.z));
    return __fadd_rn(__fadd_rn(__fmul_rn(d.x, d.x), __fmul_rn(d.y, d.y)), __fmul_rn(d.z, d.z));
}

// Production steps: a member of the 2R set (hit) adds its unit offset to the
// centrality sum here, in the sweep, and only members inside R go on to the
// queued phase (by volume the 2R set is about eight times the R set). The
// centrality sum is a float sum, compared to rounding like the forces (set
// membership never reads it), so the unit offset is d * rsqrtf(d2) (a few
// ulp) instead of a square root and three divisions; the floor 1e-12 on d2
// matches the 1e-6 floor on the distance. Returns whether the member is inside R.
__device__ __forceinline__ bool ring(Sweep& w, bool hit, const f3 d, float d2) {
    if (hit) {
        w.a.csum = add(w.a.csum, mul(d, rsqrtf(fmaxf(d2, 1e-12f))));
        w.a.n_g += 1;
    }
    return hit && d2 <= w.r2;
}

// Cheap phase over one contiguous candidate range [sc, ec) (wide paths).
template <bool SETS, bool CHECK_CELL>
__device__ __forceinline__ void sweep(Sweep& w, uint32_t sc, uint32_t ec, uint32_t lane, int cx = 0, int cy = 0,
                                      int cz = 0, float inv_cell = 0.f) {
    for (uint32_t base = sc; base < ec; base += 32) {
        const uint32_t t = base + lane;
        bool hit = false;
        if (t < ec && t != w.self) {
            const float4 q = __ldg(&w.pos[t + w.shift]);
            f3 d;
            const float d2 = offset2(w, q, d);
            hit = d2 <= w.c2;
            if (CHECK_CELL)
                hit = hit && pcell(q.x, inv_cell) == cx && pcell(q.y, inv_cell) == cy && pcell(q.z, inv_cell) == cz;
            if (!SETS) hit = ring(w, hit, d, d2);
        }
        enqueue<SETS>(w, hit, t, lane);
    }
}

// Cheap phase over the fast path's bucket ranges, packed: the ranges (one
// per lane, in lane order) are concatenated and swept 32 candidates at a time
// across range boundaries, two chunks per iteration. The candidates come in
// exactly the order of a range-by-range sweep, so the hit queue, and every
// sum, is unchanged; short ranges just stop wasting lanes. A lane finds the
// range of its candidate i from the bitmask of ranges starting in its chunk.
template <bool SETS, bool STG = false>
__device__ __forceinline__ void sweep_packed(Sweep& w, uint32_t s, uint32_t e, uint32_t lane) {
    const uint32_t nz = __ballot_sync(FULL, e > s);
    const uint32_t R = __popc(nz);
    if (!R) return;
    // lane q takes the q-th non-empty range: each non-empty lane writes its
    // range at its rank among them into the free part of the hit queue
    // (w.qn < 32 entries wait, so the 64 words from w.qn fit its 96), and lane
    // q reads entry q back
    uint32_t* scratch = w.q + w.qn;
    if (e > s) {
        const uint32_t r = __popc(nz & lanemask_lt());
        scratch[r] = s;
        scratch[32 + r] = e - s;
    }
    __syncwarp();
    const uint32_t rs = lane < R ? scratch[lane] : 0u;
    const uint32_t rl = lane < R ? scratch[32 + lane] : 0u;
    __syncwarp();
    uint32_t inc = rl;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, inc, o);
        if ((int)lane >= o) inc += y;
    }
    const uint32_t T = __shfl_sync(FULL, inc, 31);  // candidates in all
    const uint32_t P = inc - rl;                     // where this lane's range starts in the concatenation
    const uint32_t D = rs - P;                       // candidate i of this range is view index i + D
    uint32_t lemask;
    asm("mov.u32 %0, %%lanemask_le;" : "=r"(lemask));
    uint32_t r0 = 0;  // ranges started before the current chunk
    // the chunk this lane's range starts in, and its bit there (lanes >= R: none)
    const uint32_t pch = lane < R ? P >> 5 : 0xFFFFFFFFu, pbit = 1u << (P & 31u);
    for (uint32_t c0 = 0, ch = 0; c0 < T; c0 += 64, ch += 2) {
        const uint32_t bA = __reduce_or_sync(FULL, pch == ch ? pbit : 0u);
        const uint32_t bB = __reduce_or_sync(FULL, pch == ch + 1 ? pbit : 0u);
        const uint32_t iA = c0 + lane, iB = iA + 32;
        const uint32_t rA = r0 + __popc(bA & lemask) - 1;
        const uint32_t rB = r0 + __popc(bA) + __popc(bB & lemask) - 1;
        const uint32_t tA = iA + __shfl_sync(FULL, D, rA & 31), tB = iB + __shfl_sync(FULL, D, rB & 31);
        r0 += __popc(bA) + __popc(bB);
        const bool vA = iA < T && tA != w.self, vB = iB < T && tB != w.self;
        // invalid lanes read the bird's own slot (always in range) and discard it
        const float4 qA = ldpos<STG>(&w.pos[(vA ? tA : w.self) + w.shift]);
        const float4 qB = ldpos<STG>(&w.pos[(vB ? tB : w.self) + w.shift]);
        f3 dA, dB;
        const float d2A = offset2(w, qA, dA), d2B = offset2(w, qB, dB);
        bool hA = vA && d2A <= w.c2, hB = vB && d2B <= w.c2;
        if (!SETS) {
            hA = ring(w, hA, dA, d2A);
            hB = ring(w, hB, dB, d2B);
        }
        enqueue2<SETS, STG>(w, hA, tA, hB, tB, lane);
    }
}

template <bool SETS, bool STG = false>
__device__ __forceinline__ void drain(Sweep& w, uint32_t lane) {
    if (w.qn) {
        __syncwarp();
        if (lane < w.qn) take<SETS, STG>(w, w.q[lane]);
        __syncwarp();
        w.qn = 0;
    }
}

// Reduce-scatter of K = 2^m values across the warp: afterwards lane l holds the
// warp total of value index (l >> (5 - m)) & (K - 1) (fixed association). The
// float version adds value pairs with f32x2 additions (sums, not set membership).
template <int K>
__device__ __forceinline__ float rs_float(float (&v)[K], uint32_t lane) {
#pragma unroll
    for (int half = K / 2, o = 16; half >= 1; half >>= 1, o >>= 1) {
        const bool upper = (lane & o) != 0;
        if (half >= 2) {
#pragma unroll
            for (int i = 0; i < half; i += 2) {
                const float s0 = upper ? v[i] : v[i + half], s1 = upper ? v[i + 1] : v[i + 1 + half];
                const float k0 = upper ? v[i + half] : v[i], k1 = upper ? v[i + 1 + half] : v[i + 1];
                const float2 r = __fadd2_rn(make_float2(k0, k1),
                                            make_float2(__shfl_xor_sync(FULL, s0, o), __shfl_xor_sync(FULL, s1, o)));
                v[i] = r.x;
                v[i + 1] = r.y;
            }
        } else {
            const float send = upper ? v[0] : v[1];
            const float keep = upper ? v[1] : v[0];
            v[0] = __fadd_rn(keep, __shfl_xor_sync(FULL, send, o));
        }
    }
#pragma unroll
    for (int o = 16 / K; o >= 1; o >>= 1) v[0] = __fadd_rn(v[0], __shfl_xor_sync(FULL, v[0], o));
    return v[0];
}
template <int K>
__device__ __forceinline__ uint32_t rs_uint(uint32_t (&v)[K], uint32_t lane) {
#pragma unroll
    for (int half = K / 2, o = 16; half >= 1; half >>= 1, o >>= 1) {
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < half; ++i) {
            const uint32_t send = upper ? v[i] : v[i + half];
            const uint32_t keep = upper ? v[i + half] : v[i];
            v[i] = keep + __shfl_xor_sync(FULL, send, o);
        }
    }
#pragma unroll
    for (int o = 16 / K; o >= 1; o >>= 1) v[0] += __shfl_xor_sync(FULL, v[0], o);
    return v[0];
}

// params.rs:61-65 with the tabulated factor
__device__ __forceinline__ float radius_step(float r, uint32_t n, const float* __restrict__ rtab) {
    const float factor = n < (uint32_t)RADIUS_TABLE ? __ldg(&rtab[n]) : powf(__fdiv_rn(N_C, (float)n), RADIUS_EXP);
    return clampf(__fmul_rn(r, factor), R_H, R_MAX);
}

// Birds a warp batches: their search boxes are computed together
// (group_boxes, one bird per lane) and their decisions finished together (the
// epilogue, one bird per lane). Shared memory and the L1 cache share each SM's
// storage, so a smaller batch leaves decide's candidate reads more L1.
constexpr uint32_t DECIDE_BATCH = 8;

// Per-warp shared memory: the hit queue and the batch's reduced birds awaiting
// their epilogue.
template <bool SETS>
struct WarpSmem {
    static constexpr int NI = SETS ? 8 : 1;  // integer sums per bird (production steps: in red)
    int4 box[DECIDE_BATCH];          // the batch's search boxes (group_boxes)
    uint4 aux[DECIDE_BATCH];
    int2 zc[DECIDE_BATCH];           // their first cell along z and cell count along z
    uint32_t queue[96];
    float red[16][DECIDE_BATCH];     // sep xyz, coh xyz, align xyz, csum xyz (+ the four counts, production steps)
    uint32_t cnt[NI][DECIDE_BATCH];  // grid-reporting steps: n_all, n_star, n_align, n_g, the four set hashes
    uint32_t st[DECIDE_BATCH];       // slot of the bird in the reordered buffer
    uint32_t vix[DECIDE_BATCH];      // view index (set summaries)
    float pz[DECIDE_BATCH];          // height (roost pull)
};

// Search boxes of a warp's next DECIDE_BATCH deciding birds (records e,
// e + nw, ...), one bird per lane, so the box arithmetic runs once per bird
// rather than once per lane of a warp-uniform setup. Cells of edge
// 1 / inv_cell (the reference's 4 m cells in SETS steps). box: first cell x,
// y; the z-slab range floor((z -/+ reach) * 4 inv_cell) (slabs of a quarter
// cell). aux: reach^2 (f32 bits); mx | nx << 17; my | ny << 17 (multiply-shift
// constants, div_magic); the lattice bit counts (lattice_bits) | 1 << 31 when
// the box has at most 32 cells (the fast path). zc: first cell along z, cells
// along z.
template <bool SETS>
__device__ __forceinline__ void group_boxes(WarpSmem<SETS>& m, const DueRec* __restrict__ due, uint32_t e,
                                            uint32_t nw, uint32_t ndue, uint32_t lane, float inv_cell) {
    const uint32_t ej = e + lane * nw;
    if (lane < DECIDE_BATCH && ej < ndue) {
        const float4 pr = due[ej].pr;
        const uint32_t buckets = due[ej].fl.z;
        const SearchBox sb = search_box(mk(pr.x, pr.y, pr.z), pr.w, inv_cell);
        int4 box = make_int4(sb.lx, sb.ly, 0, 0);
        uint4 aux = make_uint4(__float_as_uint(sb.reach2), 0u, 0u, 0u);
        if (sb.ncell <= 32) {
            const uint32_t nx = (uint32_t)sb.nx, ny = (uint32_t)sb.ny;
            const float inv4 = __fmul_rn(4.0f, inv_cell);
            box.z = pcell(pr.z - sb.reach, inv4);
            box.w = pcell(pr.z + sb.reach, inv4);
            aux.y = div_magic(nx) | (nx << 17);
            aux.z = div_magic(ny) | (ny << 17);
            aux.w = lattice_bits(buckets) | (1u << 31);
            m.zc[lane] = make_int2(sb.lz, (int)sb.nz);
        }
        m.box[lane] = box;
        m.aux[lane] = aux;
    }
    __syncwarp();
}

// Finishes bird `slot` of the warp's batch (model.rs:95-144), one lane per bird.
template <bool SETS>
__device__ __forceinline__ void epilogue(const WarpSmem<SETS>& m, uint32_t slot, const Arena& ar,
                                         const float* __restrict__ rtab, uint32_t* __restrict__ sets) {
    const uint32_t st = m.st[slot];
    const float4* __restrict__ Bv = ar.B;
    float4* __restrict__ C = ar.C;
    float4* __restrict__ D = ar.D;
    const f3 sep = mk(m.red[0][slot], m.red[1][slot], m.red[2][slot]);
    const f3 coh = mk(m.red[3][slot], m.red[4][slot], m.red[5][slot]);
    const f3 align = mk(m.red[6][slot], m.red[7][slot], m.red[8][slot]);
    const f3 csum = mk(m.red[9][slot], m.red[10][slot], m.red[11][slot]);
    uint32_t n_all, n_star, n_align, n_g;
    if (SETS) {
        n_all = m.cnt[0][slot], n_star = m.cnt[1][slot], n_align = m.cnt[2][slot], n_g = m.cnt[3][slot];
    } else {
        n_all = __float2uint_rn(m.red[12][slot]), n_star = __float2uint_rn(m.red[13][slot]);
        n_align = __float2uint_rn(m.red[14][slot]), n_g = __float2uint_rn(m.red[15][slot]);
    }
    const f3 v = xyz(Bv[st]);
    const float4 cme = C[st];
    const float nd = D[st].x;
    const f3 fi = forward(v);
    f3 force = mk(0.f, 0.f, 0.f);
    if (n_all > 0) force = add(force, mul(sep, __fdiv_rn(W_SEP, (float)n_all)));
    const float cen = n_g > 0 ? __fdiv_rn(len(csum), (float)n_g) : 0.0f;
    if (n_star > 0) force = add(force, mul(normalize_or_zero(coh), __fmul_rn(W_COH, cen)));
    const f3 al = n_align > 0 ? sub(dvs(align, (float)n_align), fi) : mk(0.f, 0.f, 0.f);
    force = add(force, mul(al, W_ALIGN));
    const float roost = __fmul_rn(W_ROOST_V, clampf(__fdiv_rn(__fsub_rn(Z0, m.pz[slot]), H_ROOST_V), -1.0f, 1.0f));
    force = add(force, mul(mk(0.f, 0.f, 1.f), roost));
    const float speed = len(v);
    force = add(force, mul(fi, __fmul_rn(MASS / TAU, __fsub_rn(V0, speed))));
    C[st] = make_float4(force.x, force.y, force.z, radius_step(cme.w, n_all, rtab));
    D[st] = make_float4(__fadd_rn(nd, DU), __uint_as_float(n_all), cen, 0.f);
    if (SETS) {
        uint32_t* o = sets + (size_t)m.vix[slot] * 8;
#pragma unroll
        for (int k = 0; k < 8; ++k) o[k] = m.cnt[k][slot];
    }
}


// Bucket of cell (cx, cy, cz): SETS steps report their grid and use the
// reference hash; production steps use the lattice index.
template <bool SETS>
__device__ __forceinline__ uint32_t bucket_of(int cx, int cy, int cz, uint32_t buckets) {
    return SETS ? (cell_hash(cx, cy, cz) & (buckets - 1u)) : lattice_bucket(cx, cy, cz, buckets);
}

// Sets up the sweep of one deciding bird from its record.
__device__ __forceinline__ void start_bird(Sweep& w, const DueRec& rec) {
    const float r = rec.pr.w;
    w.shift = rec.fl.w;
    w.p = mk(rec.pr.x, rec.pr.y, rec.pr.z);
    w.fi = mk(rec.fk.x, rec.fk.y, rec.fk.z);
    w.r2 = __fmul_rn(r, r);
    const float rr = __fmul_rn(2.0f, r);
    w.c2 = __fmul_rn(rr, rr);
    w.self = __float_as_uint(rec.fk.w);
    w.a.sep = w.a.coh = w.a.align = w.a.csum = mk(0.f, 0.f, 0.f);
    w.a.n_all = w.a.n_star = w.a.n_align = w.a.n_g = 0;
    w.a.h_all = w.a.h_star = w.a.h_align = w.a.h_g = 0;
}

// Sweeps one deciding bird's neighbourhood from the state (record rec, its
// box from group_boxes in slot `slot` of the warp's shared memory), queueing
// and taking its hits; cells of edge `cell` (1 / inv_cell).
template <bool SETS>
__device__ __forceinline__ void sweep_bird(Sweep& w, const WarpSmem<SETS>& m, uint32_t slot, const DueRec& rec,
                                           const FlockDesc* __restrict__ fl, int nfl, uint32_t V,
                                           StepCtl* __restrict__ ctl, const uint32_t* __restrict__ offsets,
                                           const uint32_t* __restrict__ counts, const Arena& ar,
                                           const uint32_t* __restrict__ slabs, float cell, float inv_cell,
                                           uint32_t lane, uint32_t& cand) {
    const int4 box = m.box[slot];
    const uint4 aux = m.aux[slot];
    const uint32_t k = __float_as_uint(rec.fk.w), bbase = rec.fl.y, buckets = rec.fl.z;
    const float r = rec.pr.w;
    const f3 p = w.p;
    if (aux.w >> 31) {
        // fast path (search box of at most 32 cells, from group_boxes): each
        // distinct bucket of the culled box once, no cell check
        const float reach2 = __uint_as_float(aux.x);
        const uint32_t nx = aux.y >> 17, ny = aux.z >> 17;
        const int lx = box.x, ly = box.y, zlo = box.z, zhi = box.w;
        const int2 zc = m.zc[slot];
        const int lz = zc.x;
        const uint32_t ncell = nx * ny * (uint32_t)zc.y;
        bool valid = false;
        uint32_t b = 0;
        int z0 = 0, z1 = 3;  // production steps: the z-slabs of this lane's cell within reach
        if (lane < ncell) {
            // lane = ix + nx * (iy + ny * iz), quotients by multiply-shift (div_magic)
            const uint32_t t = (lane * (aux.y & 0x1FFFFu)) >> 16;
            const uint32_t iz = (t * (aux.z & 0x1FFFFu)) >> 16;
            const int cx = lx + (int)(lane - t * nx);
            const int cy = ly + (int)(t - iz * ny), cz = lz + (int)iz;
            const float ox = (float)cx * cell, oy = (float)cy * cell, oz = (float)cz * cell;
            const float dx = fminf(fmaxf(p.x, ox), ox + cell) - p.x;
            const float dy = fminf(fmaxf(p.y, oy), oy + cell) - p.y;
            const float dz = fminf(fmaxf(p.z, oz), oz + cell) - p.z;
            const float dxy2 = dx * dx + dy * dy;
            valid = dxy2 + dz * dz <= reach2;
            if (!SETS) {
                // The z-slabs of this cell that the sphere reaches: at the cell's
                // nearest xy point the sphere spans |dz| <= sqrt(reach^2 - dxy^2)
                // (dxy^2 a lower bound for any bird of the cell). The 1e-4 reach^2
                // under the root, and the reach's own absolute margin, cover the
                // rounding (and the few ulp of the reciprocal square root, the
                // argument being at least 1e-4 reach^2 > 0); the bird's whole
                // z-range zlo..zhi bounds it.
                const float hz2 = fmaxf(reach2 - dxy2, 0.f) + 1e-4f * reach2;
                const float hz = hz2 * rsqrtf(hz2);
                const float inv4 = __fmul_rn(4.0f, inv_cell);
                z0 = min(3, max(0, max(zlo, pcell(p.z - hz, inv4)) - 4 * cz));
                z1 = min(3, max(0, min(zhi, pcell(p.z + hz, inv4)) - 4 * cz));
            }
            b = bbase + (SETS ? (cell_hash(cx, cy, cz) & (buckets - 1u))
                              : lattice_bucket_bits(cx, cy, cz, aux.w));
        }
        // grid-reporting steps drop buckets shared by two cells of the box (the
        // reference hash collides); production steps have none to drop (see the
        // slab trim below: the lattice index repeats only every 16 cells or more)
        bool keep = valid;
        if (SETS) {
            const uint32_t vm = __ballot_sync(FULL, valid);
            if (valid) {
                const uint32_t peers = __match_any_sync(vm, b);
                keep = (int)lane == __ffs(peers) - 1;
            }
        }
        uint32_t s = 0, en = 0;
        if (keep) {
            // Production runs are ordered by quarter-cell z-slab within their
            // cell, and the sort left each run's slab boundaries (birds in slabs
            // < 1, < 2, < 3; 10 bits each; all ones: untrimmed). A candidate
            // within the reach has |dz| <= reach and floor is monotonic, so only
            // slabs z0..z1 of this cell can hold one: the range shrinks to them.
            // (The trim takes the bucket's cell to be this lane's: no two cells of
            // the box share a bucket in production steps, since the box spans at
            // most 3 cells per axis and the lattice index repeats only every 16
            // cells or more.)
            const uint32_t sw = SETS ? 0xFFFFFFFFu : __ldg(&slabs[b]);  // issued with the range's loads
            bucket_range(offsets, counts, b, V, w.shift, 2u * ar.cap, ctl, s, en);
            if (!SETS && en > s && sw != 0xFFFFFFFFu) {
                const uint32_t L = en - s;
                const uint32_t lo = z0 <= 0 ? 0u : (sw >> (10 * (z0 - 1))) & 1023u;
                const uint32_t hi = z1 >= 3 ? L : (sw >> (10 * z1)) & 1023u;
                if (hi <= L) {  // else a stale word: keep the run whole
                    if (lo >= hi) {
                        en = s;
                    } else {
                        en = s + hi;
                        s += lo;
                    }
                }
            }
        }
        cand += en - s;
        sweep_packed<SETS>(w, s, en, lane);
    } else {
        const SearchBox sb = search_box(p, r, inv_cell);
        const float reach2 = sb.reach2;
        const int lx = sb.lx, ly = sb.ly, lz = sb.lz;
        const long long nxl = sb.nx, nyl = sb.ny, ncell = sb.ncell;
        // the flock's own view region [vbase, vbase + n)
        const FlockDesc* fd = &fl[find_flock_v(fl, nfl, k)];
        uint32_t f0 = __ldg(&fd->vbase), f1 = f0 + __ldg(&fd->n);
        const uint32_t sf = f0 + w.shift;
        if (f1 < f0 || f1 > V || sf + (f1 - f0) < sf || sf + (f1 - f0) > 2u * ar.cap) f1 = f0 = 0;
        if (ncell * 16 >= (long long)(f1 - f0)) {
            // very wide reach: brute force over the flock's own range
            if (lane == 0) cand += f1 - f0;
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
                    const float ox = (float)cx * cell, oy = (float)cy * cell, oz = (float)cz * cell;
                    const float dx = fminf(fmaxf(p.x, ox), ox + cell) - p.x;
                    const float dy = fminf(fmaxf(p.y, oy), oy + cell) - p.y;
                    const float dz = fminf(fmaxf(p.z, oz), oz + cell) - p.z;
                    valid = dx * dx + dy * dy + dz * dz <= reach2;
                    if (valid) {
                        bucket_range(offsets, counts, bbase + bucket_of<SETS>(cx, cy, cz, buckets), V, w.shift,
                                     2u * ar.cap, ctl, s, en);
                        valid = en > s;
                    }
                }
                cand += en - s;
                uint32_t km = __ballot_sync(FULL, valid);
                while (km) {
                    const int c = __ffs(km) - 1;
                    km &= km - 1;
                    const uint32_t sc = __shfl_sync(FULL, s, c), ec = __shfl_sync(FULL, en, c);
                    const int ccx = __shfl_sync(FULL, cx, c), ccy = __shfl_sync(FULL, cy, c),
                              ccz = __shfl_sync(FULL, cz, c);
                    sweep<SETS, true>(w, sc, ec, lane, ccx, ccy, ccz, inv_cell);
                }
            }
        }
    }
    drain<SETS>(w, lane);
}

// Reduces the warp's sums for the current bird (slot `slot` of the batch, its
// slot st in the state, view index k, height pz) and runs the batch's
// epilogue once DECIDE_BATCH birds wait.
template <bool SETS>
__device__ __forceinline__ void finish_bird(Sweep& w, WarpSmem<SETS>& m, uint32_t& slot, uint32_t st, uint32_t k,
                                            float pz, const Arena& ar, const float* __restrict__ rtab,
                                            uint32_t* __restrict__ sets, uint32_t lane, uint32_t& pairs) {
    {
        // production steps carry the four counts in the float reduction's spare
        // slots: per-lane counts are small integers, so their f32 sums are exact
        float fv[16] = {w.a.sep.x,   w.a.sep.y,   w.a.sep.z,   w.a.coh.x,  w.a.coh.y,  w.a.coh.z,
                        w.a.align.x, w.a.align.y, w.a.align.z, w.a.csum.x, w.a.csum.y, w.a.csum.z,
                        SETS ? 0.f : (float)w.a.n_all, SETS ? 0.f : (float)w.a.n_star,
                        SETS ? 0.f : (float)w.a.n_align, SETS ? 0.f : (float)w.a.n_g};
        const float tf = rs_float<16>(fv, lane);
        if ((lane & 1) == 0) m.red[(lane >> 1) & 15][slot] = tf;
        if (!SETS && lane == 30) pairs += __float2uint_rn(tf);  // lane 30 holds n_g
    }
    if (SETS) {
        uint32_t iv[8] = {w.a.n_all, w.a.n_star, w.a.n_align, w.a.n_g, w.a.h_all, w.a.h_star, w.a.h_align, w.a.h_g};
        const uint32_t ti = rs_uint<8>(iv, lane);
        if ((lane & 3) == 0) m.cnt[(lane >> 2) & 7][slot] = ti;
        if (lane == 12) pairs += ti;  // lane 12 holds n_g
    }
    if (lane == 0) {
        m.st[slot] = st;
        m.vix[slot] = k;
        m.pz[slot] = pz;
    }
    if (++slot == DECIDE_BATCH) {
        __syncwarp();
        if (lane < DECIDE_BATCH) epilogue<SETS>(m, lane, ar, rtab, sets);
        __syncwarp();
        slot = 0;
    }
}

// The batch's last birds, and the per-warp counter totals (no block barrier).
template <bool SETS>
__device__ __forceinline__ void finish_warp(WarpSmem<SETS>& m, uint32_t slot, const Arena& ar,
                                            const float* __restrict__ rtab, uint32_t* __restrict__ sets,
                                            uint32_t lane, bool counts_due, uint32_t ndue, uint32_t cand,
                                            uint32_t pairs, StepCtl* __restrict__ ctl) {
    if (slot) {
        __syncwarp();
        if (lane < slot) epilogue<SETS>(m, lane, ar, rtab, sets);
    }
    const uint32_t cand_w = __reduce_add_sync(FULL, cand), pairs_w = __reduce_add_sync(FULL, pairs);
    if (lane == 0) {
        if (cand_w) atomicAdd(&ctl->cand_total, (unsigned long long)cand_w);
        if (pairs_w) atomicAdd(&ctl->pair_total, (unsigned long long)pairs_w);
        if (counts_due) atomicAdd(&ctl->due_total, (unsigned long long)ndue);
    }
}

// Dynamic shared memory: one WarpSmem<SETS> per warp. 64 registers per
// thread, so one 1024-thread CTA fills an SM; with that shape all 32 warps of
// an SM take consecutive due records, i.e. neighbouring birds, and share their
// candidates in L1 (0.221 -> 0.203 ms at 1M birds against four 256-thread
// CTAs per SM, which take records from four distant places).
template <bool SETS>
__global__ void __launch_bounds__(1024, 1) k_decide(const FlockDesc* __restrict__ fl, int nfl, uint32_t V,
                                                    StepCtl* __restrict__ ctl, const DueRec* __restrict__ due,
                                                    const uint32_t* __restrict__ offsets,
                                                    const uint32_t* __restrict__ counts, Arena ar,
                                                    const float4* __restrict__ sfwd, const float* __restrict__ rtab,
                                                    uint32_t* __restrict__ sets, const uint32_t* __restrict__ slabs,
                                                    float pcell_edge, float pinv_cell) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    WarpSmem<SETS>& m = reinterpret_cast<WarpSmem<SETS>*>(s_raw)[threadIdx.x >> 5];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t ndue = *(volatile uint32_t*)&ctl->due_count;
    uint32_t cand = 0, pairs = 0, slot = 0;

    // SETS steps: the reference's 4 m cells; production steps: the runtime edge
    const float cell = SETS ? GRID_CELL : pcell_edge, inv_cell = SETS ? INV_CELL : pinv_cell;
    Sweep w;
    w.pos = ar.A;
    w.bid = ar.id;
    w.sfwd = sfwd;
    w.q = m.queue;
    w.qn = 0;

    for (uint32_t e = gw; e < ndue; e += nw) {
        if (slot == 0) group_boxes<SETS>(m, due, e, nw, ndue, lane, inv_cell);
        const DueRec rec = due[e];  // everything the setup needs, one place
        start_bird(w, rec);
        sweep_bird<SETS>(w, m, slot, rec, fl, nfl, V, ctl, offsets, counts, ar, slabs, cell, inv_cell, lane, cand);
        finish_bird<SETS>(w, m, slot, rec.fl.x, __float_as_uint(rec.fk.w), rec.pr.z, ar, rtab, sets, lane, pairs);
    }
    finish_warp<SETS>(m, slot, ar, rtab, sets, lane, gw == 0, ndue, cand, pairs, ctl);
}

template <bool SETS>
constexpr size_t decide_smem_per_warp() {
    return sizeof(WarpSmem<SETS>);
}

}  // namespace flk
