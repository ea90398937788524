// Pass 5, cell-blocked variant (production steps): decide with the
// neighbourhood staged in shared memory by TMA bulk copies.
//
// A 1024-thread CTA takes one deciding bird per warp, 32 consecutive due
// records at a time (neighbouring birds: the sort emits them in lattice order).
// When the 32 birds belong to one flock and every bird's search box is small
// (the fast path), the CTA stages the union of their boxes: it lists the
// union's cells (at most STAGE_UMAX, fewer than 16 per axis so that no two
// share a lattice bucket), finds each cell's run of the cell-ordered state,
// lays the runs out back to back in shared memory (a block-wide scan of their
// lengths) and copies each run of positions with one `cp.async.bulk`
// (non-multicast TMA bulk copy, global -> shared) that completes on one
// mbarrier. Every run is a whole number of float4 positions at 16-byte aligned
// addresses, as the bulk copy requires. Each warp then sweeps its bird's
// cells from shared memory, with the same quarter-cell z-slab trim, packed
// sweep, hit queue and reduction as k_decide; staged positions carry their
// view index in .w, which the hit phase uses for the neighbour's heading.
// Iterations whose birds span flocks, leave the fast path or need more than
// the staging capacity sweep the state directly, as k_decide does.
//
// The mbarrier wait is bounded: one thread polls it at most STAGE_SPIN times;
// if the copies never land, the kernel records DEV_STAGE_TIMEOUT and every
// thread returns (no trap, no unbounded wait).
#pragma once

#include "k_decide.cuh"

namespace flk {

constexpr uint32_t STAGE_UMAX = 512;      // cells of a CTA's union box
constexpr uint32_t STAGE_SPIN = 1u << 22;  // mbarrier polls before giving up

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    // make the initialised barrier visible to the async (TMA) proxy
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// One arrival on the barrier that also expects `bytes` more bytes of copies.
__device__ __forceinline__ void mbar_arrive_expect(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// Non-multicast bulk copy of `bytes` (a multiple of 16) from global src to
// shared dst (both 16-byte aligned); completes `bytes` on the barrier.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// Orders this thread's earlier generic accesses to shared memory before later
// async-proxy (bulk copy) writes to it.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Per-CTA staging control block in shared memory.
struct __align__(16) StageCtl {
    unsigned long long bar;  // the copies' mbarrier
    int lo[3], hi[3];        // union box of the iteration's birds (cells)
    uint32_t bbase, buckets, shift;  // the birds' flock: bucket base, count, slot - view index
    uint32_t mixed;          // 1: birds of several flocks, or a bird off the fast path
    uint32_t total;          // positions staged
    uint32_t state;          // 0 direct, 1 staged, 2 the copies never landed
    uint32_t wsum[32];       // block scan scratch
};

// Bytes of dynamic shared memory k_decide_staged needs per CTA of `warps`
// warps with room for `cap` staged positions.
inline size_t staged_smem_bytes(int warps, uint32_t cap) {
    return (size_t)warps * sizeof(WarpSmem<false>) + sizeof(StageCtl) + STAGE_UMAX * sizeof(uint4) +
           (size_t)cap * sizeof(float4);
}

// One bird's sweep over staged cells: the fast path of sweep_bird with each
// cell's run looked up in the staging table (union box lo, dims ux, uy)
// instead of offsets/counts, and the positions read from shared memory.
__device__ __forceinline__ void sweep_bird_staged(Sweep& w, const WarpSmem<false>& m, uint32_t slot,
                                                  const DueRec& rec, const uint4* __restrict__ table,
                                                  const int (&lo)[3], int ux, int uy,
                                                  const uint32_t* __restrict__ slabs, float cell, uint32_t lane,
                                                  uint32_t& cand) {
    const int4 box = m.box[slot];
    const uint4 aux = m.aux[slot];
    const f3 p = w.p;
    const float reach2 = __uint_as_float(aux.x);
    const uint32_t nx = aux.y >> 17, ny = aux.z >> 17;
    const int lx = box.x, ly = box.y, zlo = box.z, zhi = box.w;
    const int2 zc = m.zc[slot];
    const uint32_t ncell = nx * ny * (uint32_t)zc.y;
    uint32_t s = 0, en = 0;
    if (lane < ncell) {
        const uint32_t t = (lane * (aux.y & 0x1FFFFu)) >> 16;
        const uint32_t iz = (t * (aux.z & 0x1FFFFu)) >> 16;
        const int cx = lx + (int)(lane - t * nx);
        const int cy = ly + (int)(t - iz * ny), cz = zc.x + (int)iz;
        const int z0 = min(3, max(0, zlo - 4 * cz)), z1 = min(3, max(0, zhi - 4 * cz));
        const float ox = (float)cx * cell, oy = (float)cy * cell, oz = (float)cz * cell;
        const float dx = fminf(fmaxf(p.x, ox), ox + cell) - p.x;
        const float dy = fminf(fmaxf(p.y, oy), oy + cell) - p.y;
        const float dz = fminf(fmaxf(p.z, oz), oz + cell) - p.z;
        if (dx * dx + dy * dy + dz * dz <= reach2) {
            // the cell lies in the union box (it is in this bird's box)
            const uint4 tb = table[(cx - lo[0]) + ux * ((cy - lo[1]) + uy * (cz - lo[2]))];
            if (tb.z) {
                // quarter-cell z-slab trim, as in sweep_bird
                const uint32_t sw = __ldg(&slabs[tb.w]);
                uint32_t a = 0, b = tb.z;
                if (sw != 0xFFFFFFFFu) {
                    const uint32_t L = tb.z;
                    const uint32_t l0 = z0 <= 0 ? 0u : (sw >> (10 * (z0 - 1))) & 1023u;
                    const uint32_t h0 = z1 >= 3 ? L : (sw >> (10 * z1)) & 1023u;
                    if (h0 <= L) {
                        a = l0 < h0 ? l0 : 0u;
                        b = l0 < h0 ? h0 : 0u;
                    }
                }
                s = tb.x + a;
                en = tb.x + b;
            }
        }
    }
    cand += en - s;
    sweep_packed<false, true>(w, s, en, lane);
    drain<false, true>(w, lane);
}

// Production steps, cell-blocked and staged (see the file comment). Dynamic
// shared memory: staged_smem_bytes(blockDim.x / 32, cap).
__global__ void __launch_bounds__(1024, 1) k_decide_staged(const FlockDesc* __restrict__ fl, int nfl, uint32_t V,
                                                           StepCtl* __restrict__ ctl, const DueRec* __restrict__ due,
                                                           const uint32_t* __restrict__ offsets,
                                                           const uint32_t* __restrict__ counts, Arena ar,
                                                           const float4* __restrict__ sfwd,
                                                           const float* __restrict__ rtab,
                                                           const uint32_t* __restrict__ slabs, float cell,
                                                           float inv_cell, uint32_t cap) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    const uint32_t nwarp = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WarpSmem<false>& m = reinterpret_cast<WarpSmem<false>*>(s_raw)[warp];
    StageCtl& sc = *reinterpret_cast<StageCtl*>(s_raw + nwarp * sizeof(WarpSmem<false>));
    uint4* table = reinterpret_cast<uint4*>(&sc + 1);  // per union cell: staged offset, view start, length, bucket
    float4* stage = reinterpret_cast<float4*>(table + STAGE_UMAX);
    const uint32_t gw = blockIdx.x * nwarp + warp, nw = gridDim.x * nwarp;
    const uint32_t ndue = *(volatile uint32_t*)&ctl->due_count;
    uint32_t cand = 0, pairs = 0, slot = 0, phase = 0;

    Sweep w;
    w.bid = ar.id;
    w.sfwd = sfwd;
    w.q = m.queue;
    w.qn = 0;
    if (threadIdx.x == 0) mbar_init(&sc.bar, 1);
    __syncthreads();

    // every warp runs every iteration (block barriers); a warp past the end of
    // the list has no bird
    for (uint32_t base = blockIdx.x * nwarp; base < ndue; base += nw) {
        const uint32_t e = base + warp;
        const bool has = e < ndue;
        if (threadIdx.x == 0) {
            sc.lo[0] = sc.lo[1] = sc.lo[2] = 0x7FFFFFFF;
            sc.hi[0] = sc.hi[1] = sc.hi[2] = -0x7FFFFFFF;
            sc.bbase = 0xFFFFFFFFu;
            sc.mixed = 0;
        }
        __syncthreads();
        DueRec rec;
        if (has) {
            if (slot == 0) group_boxes<false>(m, due, e, nw, ndue, lane, inv_cell);
            rec = due[e];
            if (lane == 0) {
                const int4 box = m.box[slot];
                const uint4 aux = m.aux[slot];
                const int2 zc = m.zc[slot];
                if (!(aux.w >> 31)) {
                    atomicOr(&sc.mixed, 1u);  // off the fast path
                } else {
                    atomicMin(&sc.lo[0], box.x);
                    atomicMax(&sc.hi[0], box.x + (int)(aux.y >> 17) - 1);
                    atomicMin(&sc.lo[1], box.y);
                    atomicMax(&sc.hi[1], box.y + (int)(aux.z >> 17) - 1);
                    atomicMin(&sc.lo[2], zc.x);
                    atomicMax(&sc.hi[2], zc.x + zc.y - 1);
                }
                const uint32_t old = atomicCAS(&sc.bbase, 0xFFFFFFFFu, rec.fl.y);
                if (old != 0xFFFFFFFFu && old != rec.fl.y) atomicOr(&sc.mixed, 1u);
                if (old == 0xFFFFFFFFu) {  // the first bird seen names the flock
                    sc.buckets = rec.fl.z;
                    sc.shift = rec.fl.w;
                }
            }
        }
        __syncthreads();
        // stage when the birds share a flock and their union box is small
        int ux = 0, uy = 0, uz = 0;
        const bool one = !sc.mixed && sc.bbase != 0xFFFFFFFFu;
        if (one) {
            ux = sc.hi[0] - sc.lo[0] + 1;
            uy = sc.hi[1] - sc.lo[1] + 1;
            uz = sc.hi[2] - sc.lo[2] + 1;
        }
        const bool stg = one && ux >= 1 && uy >= 1 && uz >= 1 && ux <= 15 && uy <= 15 && uz <= 15 &&
                         ux * uy * uz <= (int)STAGE_UMAX;
        const uint32_t nU = stg ? (uint32_t)(ux * uy * uz) : 0u;
        const int lo[3] = {sc.lo[0], sc.lo[1], sc.lo[2]};
        // each union cell's run, one thread per cell
        uint32_t c = 0, s0 = 0, b = 0;
        if (threadIdx.x < nU) {
            const int t = (int)threadIdx.x;
            const int cx = lo[0] + t % ux, cy = lo[1] + (t / ux) % uy, cz = lo[2] + t / (ux * uy);
            b = sc.bbase + lattice_bucket(cx, cy, cz, sc.buckets);
            uint32_t en = 0;
            bucket_range(offsets, counts, b, V, sc.shift, 2u * ar.cap, ctl, s0, en);
            c = en - s0;
        }
        // block exclusive scan of the run lengths: where each run goes
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, inc, o);
            if ((int)lane >= o) inc += y;
        }
        if (lane == 31) sc.wsum[warp] = inc;
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (uint32_t k = 0; k < nwarp; ++k) {
            const uint32_t v = sc.wsum[k];
            if (k < warp) before += v;
            total += v;
        }
        const uint32_t o = before + inc - c;
        if (threadIdx.x < nU) table[threadIdx.x] = make_uint4(o, s0, c, b);
        if (threadIdx.x == 0) sc.state = (stg && total <= cap) ? 1u : 0u;
        __syncthreads();
        const bool staged = sc.state == 1u;
        if (staged) {
            if (threadIdx.x == 0) mbar_arrive_expect(&sc.bar, total * 16u);
            __syncthreads();  // the expected bytes are registered before any copy lands
            if (threadIdx.x < nU && c) {
                fence_proxy_async_smem();  // after this iteration's and the last one's reads
                bulk_g2s(stage + o, ar.A + s0 + sc.shift, c * 16u, &sc.bar);
            }
            // one thread waits, bounded; then every thread observes the completed phase
            if (threadIdx.x == 0) {
                uint32_t polls = 0;
                bool done = mbar_test(&sc.bar, phase);
                while (!done && ++polls < STAGE_SPIN) {
                    __nanosleep(32);
                    done = mbar_test(&sc.bar, phase);
                }
                if (!done) {
                    atomicCAS(&ctl->error, 0u, (uint32_t)DEV_STAGE_TIMEOUT);
                    sc.state = 2u;
                }
            }
            __syncthreads();
            if (sc.state == 2u) {
                // give copies still in flight a second bounded wait, then every thread returns
                if (threadIdx.x == 0)
                    for (uint32_t polls = 0; polls < STAGE_SPIN && !mbar_test(&sc.bar, phase); ++polls) __nanosleep(32);
                return;
            }
            // completed already: each thread acquires the staged data (a bounded loop
            // that ends on its first test)
            for (uint32_t polls = 0; polls < STAGE_SPIN && !mbar_test(&sc.bar, phase); ++polls) {
            }
            phase ^= 1u;
            // each staged position's .w becomes its view index (headings are read by view index)
            if (threadIdx.x < nU)
                for (uint32_t j = 0; j < c; ++j) stage[o + j].w = __uint_as_float(s0 + j);
            fence_proxy_async_smem();  // these writes come before the next iteration's copies
            __syncthreads();
        }
        if (has) {
            start_bird(w, rec);
            if (staged) {
                // the bird's own cell lies in the union box: its staged index excludes it
                const f3 p = w.p;
                const int cx = pcell(p.x, inv_cell), cy = pcell(p.y, inv_cell), cz = pcell(p.z, inv_cell);
                const uint4 own = table[(cx - lo[0]) + ux * ((cy - lo[1]) + uy * (cz - lo[2]))];
                const uint32_t rel = __float_as_uint(rec.fk.w) - own.y;  // the bird within its cell's run
                w.pos = stage;
                w.shift = 0;
                w.self = rel < own.z ? own.x + rel : 0u;  // (never 0u with a consistent grid)
                sweep_bird_staged(w, m, slot, rec, table, lo, ux, uy, slabs, cell, lane, cand);
            } else {
                w.pos = ar.A;
                sweep_bird<false>(w, m, slot, rec, fl, nfl, V, ctl, offsets, counts, ar, slabs, cell, inv_cell, lane,
                                  cand);
            }
            finish_bird<false>(w, m, slot, rec.fl.x, __float_as_uint(rec.fk.w), rec.pr.z, ar, rtab, nullptr, lane,
                               pairs);
        }
        fence_proxy_async_smem();  // this iteration's reads come before the next one's copies
        __syncthreads();           // before the next iteration's staging reuses the buffers
    }
    finish_warp<false>(m, slot, ar, rtab, nullptr, lane, gw == 0, ndue, cand, pairs, ctl);
}

}  // namespace flk
