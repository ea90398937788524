// FP64 evaluation of one step from the same input state, run inside a step
// for error reports on live flocks. The same deciding birds and candidate
// cells as the f32 step; set membership, sums, forces and the flight model in
// double, in the order of operations of the oracle's FP64 twin (the reference
// model crates/flock-ref/src/model.rs:53-176 evaluated in f64). The passes run
// after the per-bucket sort, while the reordered copy still holds the input
// state, and before the f32 decide and integrate change it.
#pragma once

#include "device_common.cuh"

namespace flk {

struct d3 {
    double x, y, z;
};
__device__ __forceinline__ d3 dmk(double x, double y, double z) { return d3{x, y, z}; }
__device__ __forceinline__ d3 dadd(d3 a, d3 b) { return dmk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ d3 dsub(d3 a, d3 b) { return dmk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ d3 dmul(d3 a, double s) { return dmk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ d3 ddiv(d3 a, double s) { return dmk(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ double ddot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ d3 dcross(d3 a, d3 b) {
    return dmk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ double dlen(d3 a) { return sqrt(ddot(a, a)); }
__device__ __forceinline__ d3 dnormalize(d3 a) { return dmul(a, 1.0 / dlen(a)); }
__device__ __forceinline__ double dclamp(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }
__device__ __forceinline__ d3 dforward(d3 v) { return ddot(v, v) > 1e-12 ? dnormalize(v) : dmk(1, 0, 0); }
__device__ __forceinline__ d3 dside(d3 f) {
    const d3 s = dcross(f, dmk(0, 0, 1));
    return ddot(s, s) > 1e-8 ? dnormalize(s) : dmk(1, 0, 0);
}
__device__ __forceinline__ d3 dxyz(float4 v) { return dmk(v.x, v.y, v.z); }

// Per-lane FP64 sums of one deciding bird.
struct Acc64 {
    d3 sep, coh, align, csum;
    uint32_t n_all, n_star, n_align, n_g;
};

__device__ __forceinline__ void take64(Acc64& a, d3 p, d3 fi, double r, float4 q, float4 vq) {
    const d3 d = dsub(dxyz(q), p);
    const double d2 = ddot(d, d);
    if (d2 <= 4.0 * r * r) {
        a.csum = dadd(a.csum, ddiv(d, fmax(sqrt(d2), 1e-6)));
        a.n_g += 1;
    }
    if (d2 > r * r) return;
    const double dist = sqrt(d2);
    a.n_all += 1;
    const d3 dh = ddiv(d, fmax(dist, 1e-6));
    const double sig = (double)SIGMA;
    const double g = dist <= (double)R_H ? 1.0 : exp(-((dist - R_H) * (dist - R_H)) / (2.0 * sig * sig));
    a.sep = dsub(a.sep, dmul(dh, g));
    if (dist > (double)R_H) {
        a.coh = dadd(a.coh, dh);
        a.n_star += 1;
    }
    if (ddot(fi, dh) >= (double)BLIND_COS) {
        a.align = dadd(a.align, dforward(dxyz(vq)));
        a.n_align += 1;
    }
}

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

// One warp per deciding bird. Candidates: every distinct bucket of the
// production cells (edge `cell`) a conservative 2r box touches (the f32
// step's reach bounds every FP64 pair as well), or the flock's whole range
// when the box is wide. dec[view] receives
// steering xyz, radius, neighbour count, centrality, next decision; err[4f + 3]
// counts flock f's deciding birds.
__global__ void __launch_bounds__(256) k_decide_f64(const FlockDesc* __restrict__ fl, int nfl, uint32_t V,
                                                    StepCtl* __restrict__ ctl, const DueRec* __restrict__ due,
                                                    const uint32_t* __restrict__ offsets,
                                                    const uint32_t* __restrict__ counts, Arena ar,
                                                    double* __restrict__ dec, uint32_t* __restrict__ err, float cell,
                                                    float inv_cell) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t nd = *(volatile uint32_t*)&ctl->due_count;
    for (uint32_t e = gw; e < nd; e += nw) {
        const DueRec rec = due[e];
        const uint32_t k = __float_as_uint(rec.fk.w), st = rec.fl.x, bbase = rec.fl.y, buckets = rec.fl.z,
                       shift = rec.fl.w;
        const float4 a_me = ar.A[st], b_me = ar.B[st], c_me = ar.C[st], d_me = ar.D[st];
        const d3 p = dxyz(a_me);
        const double r = c_me.w;
        const d3 fi = dforward(dxyz(b_me));
        const float rf = c_me.w;
        const float rr = __fmul_rn(2.0f, rf);
        const float pm = fmaxf(fabsf(a_me.x), fmaxf(fabsf(a_me.y), fabsf(a_me.z)));
        const float reach = rr * 1.00001f + 1e-3f + pm * 1e-6f;
        const float reach2 = reach * reach;
        const int lx = pcell(a_me.x - reach, inv_cell), ly = pcell(a_me.y - reach, inv_cell),
                  lz = pcell(a_me.z - reach, inv_cell);
        const long long nxl = (long long)pcell(a_me.x + reach, inv_cell) - lx + 1,
                        nyl = (long long)pcell(a_me.y + reach, inv_cell) - ly + 1,
                        nzl = (long long)pcell(a_me.z + reach, inv_cell) - lz + 1;
        const bool wide = nxl > (1 << 20) || nyl > (1 << 20) || nzl > (1 << 20);
        const long long ncell = wide ? (1ll << 62) : nxl * nyl * nzl;
        Acc64 acc;
        acc.sep = acc.coh = acc.align = acc.csum = dmk(0, 0, 0);
        acc.n_all = acc.n_star = acc.n_align = acc.n_g = 0;
        if (ncell <= 32) {
            bool valid = false;
            uint32_t b = 0;
            if ((long long)lane < ncell) {
                const int nx = (int)nxl, ny = (int)nyl;
                const int cx = lx + (int)lane % nx;
                const int t = (int)lane / nx;
                const int cy = ly + t % ny, cz = lz + t / ny;
                const float ox = (float)cx * cell, oy = (float)cy * cell, oz = (float)cz * cell;
                const float dx = fminf(fmaxf(a_me.x, ox), ox + cell) - a_me.x;
                const float dy = fminf(fmaxf(a_me.y, oy), oy + cell) - a_me.y;
                const float dz = fminf(fmaxf(a_me.z, oz), oz + cell) - a_me.z;
                valid = dx * dx + dy * dy + dz * dz <= reach2;
                b = bbase + lattice_bucket(cx, cy, cz, buckets);
            }
            const uint32_t vm = __ballot_sync(FULL, valid);
            bool keep = false;
            if (valid) {
                const uint32_t peers = __match_any_sync(vm, b);
                keep = (int)lane == __ffs(peers) - 1;
            }
            uint32_t s = 0, en = 0;
            if (keep) {
                const uint32_t c = __ldg(&counts[b]);
                s = __ldg(&offsets[b]);
                en = s + c;
                const uint32_t ss = s + shift;
                if (c == 0 || en < s || en > V || ss + c < ss || ss + c > 2u * ar.cap) en = s = 0;
            }
            uint32_t km = __ballot_sync(FULL, en > s);
            while (km) {
                const int c = __ffs(km) - 1;
                km &= km - 1;
                const uint32_t sc = __shfl_sync(FULL, s, c), ec = __shfl_sync(FULL, en, c);
                for (uint32_t t = sc + lane; t < ec; t += 32)
                    if (t != k) take64(acc, p, fi, r, ar.A[t + shift], ar.B[t + shift]);
            }
        } else {
            const FlockDesc* fd = &fl[find_flock_v(fl, nfl, k)];
            uint32_t f0 = __ldg(&fd->vbase), f1 = f0 + __ldg(&fd->n);
            const uint32_t sf = f0 + shift;
            if (f1 < f0 || f1 > V || sf + (f1 - f0) < sf || sf + (f1 - f0) > 2u * ar.cap) f1 = f0 = 0;
            for (uint32_t t = f0 + lane; t < f1; t += 32)
                if (t != k) take64(acc, p, fi, r, ar.A[t + shift], ar.B[t + shift]);
        }
        const d3 sep = dmk(wsum(acc.sep.x), wsum(acc.sep.y), wsum(acc.sep.z));
        const d3 coh = dmk(wsum(acc.coh.x), wsum(acc.coh.y), wsum(acc.coh.z));
        const d3 align = dmk(wsum(acc.align.x), wsum(acc.align.y), wsum(acc.align.z));
        const d3 csum = dmk(wsum(acc.csum.x), wsum(acc.csum.y), wsum(acc.csum.z));
        const uint32_t n_all = __reduce_add_sync(FULL, acc.n_all), n_star = __reduce_add_sync(FULL, acc.n_star),
                       n_align = __reduce_add_sync(FULL, acc.n_align), n_g = __reduce_add_sync(FULL, acc.n_g);
        if (lane == 0) {
            d3 force = dmk(0, 0, 0);
            if (n_all) force = dadd(force, dmul(sep, (double)W_SEP / n_all));
            const double cen = n_g ? dlen(csum) / n_g : 0.0;
            if (n_star) {
                const double l = dlen(coh);
                if (l > 0) force = dadd(force, dmul(coh, (double)W_COH * cen / l));
            }
            if (n_align) force = dadd(force, dmul(dsub(ddiv(align, n_align), fi), (double)W_ALIGN));
            force.z += (double)W_ROOST_V * dclamp(((double)Z0 - p.z) / (double)H_ROOST_V, -1, 1);
            force = dadd(force, dmul(fi, ((double)MASS / (double)TAU) * ((double)V0 - dlen(dxyz(b_me)))));
            const double nn = n_all > 1 ? n_all : 1;
            double* o = dec + (size_t)k * 8;
            o[0] = force.x;
            o[1] = force.y;
            o[2] = force.z;
            o[3] = dclamp(r * pow((double)N_C / nn, (double)RADIUS_LERP / 3.0), (double)R_H, (double)R_MAX);
            o[4] = n_all;
            o[5] = cen;
            o[6] = (double)d_me.x + (double)DU;
            atomicAdd(&err[4 * find_flock_v(fl, nfl, k) + 3], 1u);
        }
    }
}

// Every bird: the FP64 flight step from the input state and, for deciding
// birds, the FP64 decision; out[view * 15 + w] in .flk word order.
__global__ void __launch_bounds__(256) k_integrate_f64(const FlockDesc* __restrict__ fl, int nfl, uint32_t V,
                                                       Arena ar, const double* __restrict__ dec,
                                                       double* __restrict__ out) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        const FlockDesc* d = &fl[find_flock_v(fl, nfl, v)];
        if (!d->remaining) continue;
        const uint32_t st = v + view_shift(d->sbase, d->vbase, d->parity ^ 1u, ar.cap);
        const float4 a = ar.A[st], b = ar.B[st], c = ar.C[st], e = ar.D[st];
        const float t_now = __fadd_rn(d->time, DT);
        d3 steer = dxyz(c);
        double radius = c.w, next = e.x, nb = __float_as_uint(e.y), cen = e.z;
        if (t_now >= e.x) {
            const double* o = dec + (size_t)v * 8;
            steer = dmk(o[0], o[1], o[2]);
            radius = o[3];
            nb = o[4];
            cen = o[5];
            next = o[6];
        }
        const double dt = DT, mass = MASS, g = G, v0 = V0;
        d3 vel = dxyz(b);
        const d3 f = dforward(vel), side = dside(f);
        const double speed = fmax(dlen(vel), 1e-6);
        const double a_lat = ddot(steer, side) / mass;
        const double maxb = 80.0 * 3.14159265358979323846 / 180.0;
        const double target = dclamp(atan(a_lat / g), -maxb, maxb);
        const double rate = dclamp((target - (double)a.w) / (double)TAU_ROLL, -(double)MAX_ROLL_RATE,
                                   (double)MAX_ROLL_RATE);
        const double beta = dclamp((double)a.w + rate * dt, -maxb, maxb);
        const d3 up0 = dcross(side, f);
        const d3 up = dadd(dmul(up0, cos(beta)), dmul(side, sin(beta)));
        const double cb = fmax(cos(beta), 0.2), sr = speed / v0;
        const double lift = sr * sr * (double)L0 / cb, drag = sr * sr * (double)D0;
        d3 flight = dadd(dsub(dmul(up, lift), dmul(f, drag)), dmul(f, (double)D0));
        flight.z -= mass * g;
        const d3 control = dsub(steer, dmul(side, ddot(steer, side)));
        vel = dadd(vel, dmul(ddiv(dadd(control, flight), mass), dt));
        const double sp = dlen(vel);
        if (sp > 2.0 * v0) vel = dmul(vel, 2.0 * v0 / sp);
        else if (sp < 0.5 * v0 && sp > 1e-6) vel = dmul(vel, 0.5 * v0 / sp);
        const d3 pos = dadd(dxyz(a), dmul(vel, dt));
        double* w = out + (size_t)v * 15;
        w[0] = pos.x; w[1] = pos.y; w[2] = pos.z;
        w[3] = vel.x; w[4] = vel.y; w[5] = vel.z;
        w[6] = beta; w[7] = rate; w[8] = radius;
        w[9] = steer.x; w[10] = steer.y; w[11] = steer.z;
        w[12] = next; w[13] = nb; w[14] = cen;
    }
}

// After the f32 step: per bird the relative error of position and velocity
// (||f32 - f64|| / max(||f64||, 1e-6)) and whether the neighbour counts
// differ, reduced per flock f of the table: err[4f], err[4f + 1] maxima as
// float bits, err[4f + 2] mismatches. active[f]: flock f was stepped (its
// parity is flipped by now). The loop is warp-uniform; lanes of one flock
// reduce together (match_any) and their first lane updates the flock's words.
__global__ void __launch_bounds__(256) k_compare_f64(const FlockDesc* __restrict__ fl, int nfl, uint32_t V,
                                                     Arena ar, const uint8_t* __restrict__ active,
                                                     const double* __restrict__ out, uint32_t* __restrict__ err) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t blk = blockIdx.x * blockDim.x; blk < V; blk += stride) {
        const uint32_t v = blk + threadIdx.x;
        int f = -1;
        float mp = 0.f, mv = 0.f;
        uint32_t mism = 0;
        if (v < V) {
            f = find_flock_v(fl, nfl, v);
            if (active[f]) {
                const FlockDesc* d = &fl[f];
                const uint32_t st = v + view_shift(d->sbase, d->vbase, d->parity, ar.cap);
                const double* w = out + (size_t)v * 15;
                const float4 a = ar.A[st], b = ar.B[st];
                const float nb = ar.D[st].y;
                const d3 dp = dsub(dxyz(a), dmk(w[0], w[1], w[2])), dv = dsub(dxyz(b), dmk(w[3], w[4], w[5]));
                mp = (float)(dlen(dp) / fmax(dlen(dmk(w[0], w[1], w[2])), 1e-6));
                mv = (float)(dlen(dv) / fmax(dlen(dmk(w[3], w[4], w[5])), 1e-6));
                mism = (double)__float_as_uint(nb) != w[13];
            } else {
                f = -1;
            }
        }
        const uint32_t peers = __match_any_sync(FULL, f);
        // non-negative floats order as their bits
        const uint32_t bp = __reduce_max_sync(peers, __float_as_uint(mp));
        const uint32_t bv = __reduce_max_sync(peers, __float_as_uint(mv));
        const uint32_t bm = __reduce_add_sync(peers, mism);
        if (f >= 0 && (int)lane == __ffs(peers) - 1) {
            atomicMax(&err[4 * f], bp);
            atomicMax(&err[4 * f + 1], bv);
            if (bm) atomicAdd(&err[4 * f + 2], bm);
        }
    }
}

}  // namespace flk
