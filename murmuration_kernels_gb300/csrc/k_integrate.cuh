// Pass 6: integrate (reference crates/flock-ref/src/model.rs:149-176;
// cuda/flock.cu:293-328) and the end-of-step bookkeeping.
#pragma once

#include "device_common.cuh"
#include "k_grid.cuh"

namespace flk {

// One bird's flight step (model.rs:149-176): the roll follows the bank the
// lateral steering asks for, then lift, drag, gravity and the control force
// change the velocity, the speed is clamped and the position advances.
// a = position, roll; bv = velocity, spin; c = steering, radius; na, nb get
// the new A and B words. Position, velocity, roll and spin are held to a
// tolerance (1e-5 relative per bird against the oracle), not bit for bit; the
// exact words (next decision, neighbour count, radius) come from decide. So
// the pass uses the cheap forms that tolerance allows: reciprocal square
// roots for the norms, fast sine/cosine (|beta| <= MAX_BANK) and division, and
// constant divisors folded into multiplications. The pass is issue-bound, so
// its instruction count sets its time.
__device__ __forceinline__ void fly(const float4 a, const float4 bv, const float4 c, float4& na, float4& nb) {
    constexpr float INV_MASS_G = 1.0f / (MASS * G);
    constexpr float INV_TAU_ROLL = 1.0f / TAU_ROLL;
    constexpr float INV_V0 = 1.0f / V0;
    constexpr float DT_MASS = DT / MASS;
    f3 vel = xyz(bv);
    const f3 steering = xyz(c);
    const float roll = a.w;
    // forward(vel) and |vel|
    const float vv = dot(vel, vel);
    const float ivl = rsqrtf(vv);
    const float vlen = vv > 0.f ? __fmul_rn(vv, ivl) : 0.f;
    const f3 fw = vv > 1e-12f ? mul(vel, ivl) : mk(1.f, 0.f, 0.f);
    // side_of(fw): cross(fw, z) = (fw.y, -fw.x, 0), normalised
    const float s2 = __fadd_rn(__fmul_rn(fw.x, fw.x), __fmul_rn(fw.y, fw.y));
    const f3 side = s2 > 1e-8f ? mul(mk(fw.y, -fw.x, 0.f), rsqrtf(s2)) : mk(1.f, 0.f, 0.f);
    const float speed = fmaxf(vlen, 1e-6f);
    const float ss = dot(steering, side);
    const float target = clampf(atanf(__fmul_rn(ss, INV_MASS_G)), -MAX_BANK, MAX_BANK);
    const float rate = clampf(__fmul_rn(__fsub_rn(target, roll), INV_TAU_ROLL), -MAX_ROLL_RATE, MAX_ROLL_RATE);
    const float beta = clampf(__fadd_rn(roll, __fmul_rn(rate, DT)), -MAX_BANK, MAX_BANK);
    float sb, cb;
    __sincosf(beta, &sb, &cb);
    // body_up(fw, beta) = cross(side, fw) cos(beta) + side sin(beta), side.z = 0
    const f3 up0 = mk(__fmul_rn(side.y, fw.z), -__fmul_rn(side.x, fw.z),
                      __fsub_rn(__fmul_rn(side.x, fw.y), __fmul_rn(fw.x, side.y)));
    const f3 up = add(mul(up0, cb), mul(side, sb));
    const float cos_beta = fmaxf(cb, 0.2f);
    const float sr = __fmul_rn(speed, INV_V0);
    const float sr2 = __fmul_rn(sr, sr);
    const float lift = __fdividef(__fmul_rn(sr2, L0), cos_beta);
    const float drag = __fmul_rn(sr2, D0);
    const f3 flight = sub(add(sub(mul(up, lift), mul(fw, drag)), mul(fw, D0)), mk(0.f, 0.f, __fmul_rn(MASS, G)));
    const f3 control = sub(steering, mul(side, ss));
    vel = add(vel, mul(add(control, flight), DT_MASS));
    const float sp2 = dot(vel, vel);
    const float isp = rsqrtf(sp2);
    const float sp = sp2 > 0.f ? __fmul_rn(sp2, isp) : 0.f;
    if (sp > V_MAX) {
        vel = mul(vel, __fmul_rn(V_MAX, isp));
    } else if (sp < V_MIN && sp > 1e-6f) {
        vel = mul(vel, __fmul_rn(V_MIN, isp));
    }
    const f3 pos = add(xyz(a), mul(vel, DT));
    na = make_float4(pos.x, pos.y, pos.z, beta);
    nb = make_float4(vel.x, vel.y, vel.z, rate);
}

// ---------------------------------------------------------------------------
// pass 6: integrate (model.rs:149-176) + end-of-step bookkeeping
// ---------------------------------------------------------------------------
// Works on the buffer the sort pass wrote (parity ^ 1); the last block makes
// that buffer current. Clears this step's histogram entries (grid buffer cur).
// FUSE (production runs of several steps): also counts the next step's grid
// from the new positions into grid buffer nxt (key, arrival rank, histogram)
// for every flock that steps again, so the next step needs no separate hash
// pass; the counting is count_block, as in k_hash_count<true> (production
// cells of edge 1 / inv_cell).
template <bool FUSE>
__global__ void __launch_bounds__(256) k_integrate(FlockDesc* __restrict__ fl, int nfl, uint32_t V, Arena ar,
                                                   GridBuf cur, GridBuf nxt, uint32_t* __restrict__ key,
                                                   uint32_t* __restrict__ arrival, StepCtl* __restrict__ ctl,
                                                   float inv_cell) {
    __shared__ uint32_t s_first[2][8];
    // the histogram's occupied entries go back to zero for the step after next
    const uint32_t nocc = *(volatile const uint32_t*)cur.occ_count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nocc; i += gridDim.x * blockDim.x)
        cur.counts[cur.occ[i]] = 0;
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t it = 0;
    for (uint32_t blk = blockIdx.x * blockDim.x; blk < V; blk += stride, it ^= 1u) {
        const uint32_t v = blk + threadIdx.x;
        bool act = false;
        uint32_t b = 0, slab = 0;
        if (v < V) {
            const FlockDesc* d = &fl[find_flock_v(fl, nfl, v)];
            const uint32_t rem = d->remaining;
            if (rem) {
                float4* __restrict__ A = ar.A;
                float4* __restrict__ B = ar.B;
                const float4* __restrict__ C = ar.C;
                const uint32_t st = v + view_shift(d->sbase, d->vbase, d->parity ^ 1u, ar.cap);
                const float4 a = A[st];
                const float4 bv = B[st];
                const float4 c = C[st];
                float4 na, nb;
                fly(a, bv, c, na, nb);
                A[st] = na;
                B[st] = nb;
                if (FUSE && rem >= 2) {  // this flock steps again: its bird's cell for the next step
                    b = bucket_slab<true>(na, d->bbase, d->buckets, slab,
                                          inv_cell, __fmul_rn(4.0f, inv_cell));
                    key[v] = b;
                    act = true;
                }
            }
        }
        if (FUSE) count_block<false>(act, v, b, slab, arrival, nxt, ctl, s_first, it);
    }
    // the last block to finish advances every active flock and resets the step counters
    __shared__ bool s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&ctl->done_blocks, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        for (int f = threadIdx.x; f < nfl; f += blockDim.x) {
            fl[f].cursor = 0;
            if (fl[f].remaining) {
                fl[f].time = __fadd_rn(fl[f].time, DT);
                fl[f].remaining -= 1;
                fl[f].parity ^= 1u;
            }
        }
        if (threadIdx.x == 0) {
            *cur.occ_count = 0;
            ctl->due_count = 0;
            ctl->scan_ticket = 0;
            ctl->scan_skip1 = 0;  // the scan test hook lasts one step
            ctl->scan_spin = 0;
            ctl->epoch = ctl->epoch + 1;
            ctl->done_blocks = 0;
        }
    }
}


}  // namespace flk
