// Passes 1-4 of the step: .flk words <-> arena, cell key + histogram, the
// single-pass decoupled look-back scan, scatter by arrival rank, and the
// per-bucket stable sort that moves each flock's state into cell order and
// writes the deciding-bird list (reference cuda/flock.cu:118-179, made stable).
//
// A flock's state lives in one of two buffers (FlockDesc::parity). A step
// reads it from buffer parity, in the cell order of the previous step, and
// the sort writes it to buffer parity ^ 1 in this step's cell order; decide
// and integrate then work on that copy, and integrate's last block flips the
// parity. Because consecutive slots already hold birds of one cell, the
// histogram's atomics aggregate within a warp, the scatter writes runs, and
// the sort's gathers read mostly contiguous runs.
#pragma once

#include "device_common.cuh"

namespace flk {


// ---------------------------------------------------------------------------
// .flk words <-> arena (A = pos,roll  B = vel,spin  C = steer,radius  D = next,nb,cen)
// ---------------------------------------------------------------------------
// Loads bird i of a flock into slot base + i (bird order).
__global__ void k_unpack(const float* __restrict__ w, uint32_t n, uint32_t base, Arena s) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* r = w + (size_t)i * WORDS;
        const uint32_t k = base + i;
        s.A[k] = make_float4(r[0], r[1], r[2], r[6]);
        s.B[k] = make_float4(r[3], r[4], r[5], r[7]);
        s.C[k] = make_float4(r[9], r[10], r[11], r[8]);
        s.D[k] = make_float4(r[12], r[13], r[14], 0.f);
        s.id[k] = i;
    }
}

// Writes the flock held in slots [base, base + n) (any order) back as .flk
// words in bird order.
__global__ void k_pack(float* __restrict__ w, uint32_t n, uint32_t base, Arena s) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = base + i;
        const uint32_t bird = s.id[k];
        if (bird >= n) continue;  // never for a valid arena
        float* r = w + (size_t)bird * WORDS;
        const float4 a = s.A[k], b = s.B[k], c = s.C[k], d = s.D[k];
        r[0] = a.x; r[1] = a.y; r[2] = a.z;
        r[3] = b.x; r[4] = b.y; r[5] = b.z;
        r[6] = a.w; r[7] = b.w; r[8] = c.w;
        r[9] = c.x; r[10] = c.y; r[11] = c.z;
        r[12] = d.x; r[13] = d.y; r[14] = d.z;
    }
}

// ---------------------------------------------------------------------------
// pass 1: cell key + histogram (warp-aggregated atomics)
// ---------------------------------------------------------------------------
// Counts one CTA iteration of birds into grid buffer g: a thread's bird v
// (act) falls in bucket b, z-slab `slab`. Bucket counts use one atomic per
// run of adjacent lanes with one bucket and give each bird its arrival rank
// (slab in the top two bits). APPEND (grid-reporting steps): the occupied-bucket list gets
// one atomic per CTA iteration (the first-seen buckets of all eight warps are
// placed from a shared-memory prefix), so the single list counter is not hit
// once per warp; production steps list the occupied buckets in k_place
// instead. Called by all threads of a 256-thread CTA; `it` alternates the
// shared slots between iterations.
template <bool APPEND>
__device__ __forceinline__ void count_block(bool act, uint32_t v, uint32_t b, uint32_t slab,
                                            uint32_t* __restrict__ arrival, const GridBuf& g,
                                            StepCtl* __restrict__ ctl, uint32_t (&s_first)[2][8], uint32_t it) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // Birds come in cell order, so equal buckets sit in runs of adjacent lanes:
    // each maximal run of active lanes with one bucket takes one atomic (its
    // first lane's) for the run's length, and lane k of the run gets rank
    // old + k. A bucket that recurs after a gap takes another atomic; ranks stay
    // distinct, and the sort orders every run by bird, so results do not
    // depend on them.
    const uint32_t m = __ballot_sync(FULL, act);
    const uint32_t bp = __shfl_up_sync(FULL, b, 1), bn = __shfl_down_sync(FULL, b, 1);
    const bool head = act && (lane == 0 || !((m >> (lane - 1)) & 1u) || bp != b);
    const bool tail = act && (lane == 31 || !((m >> (lane + 1)) & 1u) || bn != b);
    const uint32_t H = __ballot_sync(FULL, head), E = __ballot_sync(FULL, tail);
    uint32_t le;
    asm("mov.u32 %0, %%lanemask_le;" : "=r"(le));
    const uint32_t h = 31u - (uint32_t)__clz(H & le);  // this lane's run head (active lanes)
    uint32_t old = 0;
    if (head) old = atomicAdd(&g.counts[b], (uint32_t)__ffs(E >> lane));  // the run ends at lane + len - 1
    old = __shfl_sync(FULL, old, act ? h : lane);
    bool first = false;
    if (act) {
        const uint32_t rank = old + (lane - h);
        if (rank >= (1u << 30)) atomicCAS(&ctl->error, 0u, (uint32_t)DEV_BAD_RANGE);  // 2^30 birds in one cell
        arrival[v] = (rank & 0x3FFFFFFFu) | (slab << 30);
        first = rank == 0;
    }
    if (!APPEND) return;
    const uint32_t fm = __ballot_sync(FULL, first);
    if (lane == 0) s_first[it][warp] = __popc(fm);
    __syncthreads();
    if (threadIdx.x < 32) {
        // warp 0: exclusive prefix over the eight warps + one atomic
        const uint32_t c = lane < 8 ? s_first[it][lane] : 0u;
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, inc, o);
            if ((int)lane >= o) inc += y;
        }
        const uint32_t total = __shfl_sync(FULL, inc, 7);
        uint32_t base = 0;
        if (lane == 0 && total) base = atomicAdd(g.occ_count, total);
        base = __shfl_sync(FULL, base, 0);
        if (lane < 8) s_first[it][lane] = base + inc - c;
    }
    __syncthreads();
    if (first) g.occ[s_first[it][warp] + __popc(fm & lanemask_lt())] = b;
}

// Cell of position p as its bucket (LATTICE: lattice_bucket of the
// production cell of edge 1 / inv_cell; otherwise the reference's 4 m cell
// and hash, whose keys a grid-reporting step returns) and, in production
// steps, its quarter-cell z-slab within the cell (inv4 = 4 * inv_cell).
template <bool LATTICE>
__device__ __forceinline__ uint32_t bucket_slab(const float4 p, uint32_t bbase, uint32_t nb, uint32_t& slab,
                                                float inv_cell, float inv4) {
    if (!LATTICE) {
        slab = 0u;
        return bbase + (cell_hash(cell1(p.x), cell1(p.y), cell1(p.z)) & (nb - 1u));
    }
    const int cx = pcell(p.x, inv_cell), cy = pcell(p.y, inv_cell), cz = pcell(p.z, inv_cell);
    slab = pslab(p.z, cz, inv4);
    return bbase + lattice_bucket(cx, cy, cz, nb);
}

// LATTICE: a production step, whose sort orders each run by z-slab (the slab
// rides in the arrival rank); otherwise a grid-reporting step (slab 0 for
// every bird). Each CTA takes 256 consecutive view indices per iteration.
template <bool LATTICE>
__global__ void __launch_bounds__(256) k_hash_count(const FlockDesc* __restrict__ fl, int nfl, uint32_t V,
                                                    Arena ar, uint32_t* __restrict__ key,
                                                    uint32_t* __restrict__ arrival, GridBuf g,
                                                    StepCtl* __restrict__ ctl, float inv_cell) {
    __shared__ uint32_t s_first[2][8];  // per warp: first-seen buckets, then their start in occ
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t it = 0;
    for (uint32_t blk = blockIdx.x * blockDim.x; blk < V; blk += stride, it ^= 1u) {
        const uint32_t v = blk + threadIdx.x;
        bool act = false;
        uint32_t b = 0, slab = 0;
        if (v < V) {
            const FlockDesc* d = &fl[find_flock_v(fl, nfl, v)];
            if (__ldg(&d->remaining)) {
                const float4 p = ar.A[v + view_shift(__ldg(&d->sbase), __ldg(&d->vbase), __ldg(&d->parity), ar.cap)];
                b = bucket_slab<LATTICE>(p, __ldg(&d->bbase), __ldg(&d->buckets), slab, inv_cell,
                                         __fmul_rn(4.0f, inv_cell));
                key[v] = b;
                act = true;
            }
        }
        count_block<!LATTICE>(act, v, b, slab, arrival, g, ctl, s_first, it);
    }
}

// ---------------------------------------------------------------------------
// pass 2: single-pass decoupled look-back exclusive scan (counts -> offsets)
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long scan_word(uint32_t epoch, uint32_t flag, uint32_t value) {
    return ((unsigned long long)(epoch & 0x3FFFFFFFu) << 34) | ((unsigned long long)flag << 32) | value;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan(const uint32_t* __restrict__ counts, uint32_t* __restrict__ offsets,
                                                       uint32_t ntiles, unsigned long long* __restrict__ status,
                                                       StepCtl* __restrict__ ctl) {
    __shared__ uint32_t s_tile, s_prefix;
    __shared__ uint32_t s_warp[SCAN_THREADS / 32];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_tile = atomicAdd(&ctl->scan_ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) {  // only after an aborted step left the ticket counter off
        if (threadIdx.x == 0) atomicCAS(&ctl->error, 0u, (uint32_t)DEV_BAD_RANGE);
        return;
    }
    const uint32_t epoch = *(volatile uint32_t*)&ctl->epoch & 0x3FFFFFFFu;
    const size_t base = (size_t)tile * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
    // test hook (normally 0 / 0): a tile that publishes nothing, a shorter poll limit
    const bool publish = tile + 1u != *(volatile uint32_t*)&ctl->scan_skip1;
    const uint32_t spin = *(volatile uint32_t*)&ctl->scan_spin;
    const uint32_t spin_limit = spin ? spin : SCAN_SPIN_LIMIT;

    uint4 c[SCAN_ITEMS / 4];
    const uint4* src = reinterpret_cast<const uint4*>(counts + base);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS / 4; ++k) c[k] = src[k];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS / 4; ++k) sum += c[k].x + c[k].y + c[k].z + c[k].w;

    // block exclusive scan of the per-thread sums
    uint32_t inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, inc, o);
        if ((int)lane >= o) inc += y;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    uint32_t wpre = 0, agg = 0;
#pragma unroll
    for (int w = 0; w < SCAN_THREADS / 32; ++w) {
        const uint32_t t = s_warp[w];
        if (w < (int)warp) wpre += t;
        agg += t;
    }
    const uint32_t texcl = wpre + inc - sum;

    if (warp == 0) {
        uint32_t excl = 0;
        if (tile == 0) {
            if (lane == 0 && publish) st_relaxed(&status[0], scan_word(epoch, FLAG_P, agg));
        } else {
            if (lane == 0 && publish) st_relaxed(&status[tile], scan_word(epoch, FLAG_A, agg));
            int pred = (int)tile - 1;
            uint32_t polls = 0;
            while (true) {
                const int idx = pred - (int)lane;
                uint32_t flag = FLAG_P, val = 0;
                while (true) {
                    if (idx >= 0) {
                        const unsigned long long w = ld_relaxed(&status[idx]);
                        const bool ok = (uint32_t)(w >> 34) == epoch;
                        flag = ok ? (uint32_t)((w >> 32) & 3u) : 0u;
                        val = (uint32_t)w;
                    }
                    if (__all_sync(FULL, flag != 0)) break;
                    if (++polls > spin_limit) {  // give up: record and let every waiter finish
                        if (lane == 0) atomicCAS(&ctl->error, 0u, (uint32_t)DEV_SCAN_TIMEOUT);
                        flag = FLAG_P;
                        val = 0;
                        break;
                    }
                    __nanosleep(64);
                }
                const uint32_t pm = __ballot_sync(FULL, flag == FLAG_P);
                const int firstp = pm ? __ffs(pm) - 1 : 32;
                uint32_t x = ((int)lane <= firstp) ? val : 0u;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
                excl += x;
                if (pm) break;
                pred -= 32;
            }
            if (lane == 0 && publish) st_relaxed(&status[tile], scan_word(epoch, FLAG_P, excl + agg));
        }
        if (lane == 0) s_prefix = excl;
    }
    __syncthreads();
    uint32_t run = s_prefix + texcl;
    uint4* dst = reinterpret_cast<uint4*>(offsets + base);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS / 4; ++k) {
        uint4 o;
        o.x = run; run += c[k].x;
        o.y = run; run += c[k].y;
        o.z = run; run += c[k].z;
        o.w = run; run += c[k].w;
        dst[k] = o;
    }
    if (tile == ntiles - 1 && threadIdx.x == SCAN_THREADS - 1) offsets[(size_t)ntiles * SCAN_TILE] = run;
}

// ---------------------------------------------------------------------------
// pass 2' (steps without grid output): list and place the occupied buckets
// ---------------------------------------------------------------------------
// Production steps need each occupied bucket's birds contiguous, not the dense
// canonical offsets. Each warp reads the histogram 128 consecutive buckets at
// a time (four per lane). A flock's buckets are a power of two, at least
// 2^12, so every flock's range starts at a multiple of 2^12 and the window
// lies in one flock. Its occupied buckets get run starts inside the flock's
// view region [vbase, vbase + n) from the flock's cursor and places in the
// occupied-bucket list, one atomicAdd on each per window (warp prefix sums in
// between). The list thus holds lattice rows: consecutive buckets are
// neighbouring cells along x, so the sort's contiguous bucket ranges, and the
// deciding birds taken from them in order, are spatial neighbours whose
// candidates decide's warps share in L1. Where a run lands does not change
// any result: decide visits buckets in cell order and each run in (slab,
// bird) order. The start is written to offsets[b]; the bucket's length stays
// in counts[b] until integrate clears it.
__global__ void __launch_bounds__(256) k_place(FlockDesc* __restrict__ fl, int nfl, uint32_t nb,
                                               const uint32_t* __restrict__ counts, uint32_t* __restrict__ offsets,
                                               uint32_t* __restrict__ occ, uint32_t* __restrict__ occ_count) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i0 = gw * 128u; i0 < nb; i0 += nw * 128u) {
        const uint32_t b0 = i0 + 4u * lane;  // nb is a multiple of 2^12: the four lie inside
        const uint4 c = reinterpret_cast<const uint4*>(counts)[b0 >> 2];
        const uint32_t n_occ = (c.x != 0) + (c.y != 0) + (c.z != 0) + (c.w != 0);
        if (!__any_sync(FULL, n_occ != 0)) continue;  // warp-uniform
        const uint32_t n_birds = c.x + c.y + c.z + c.w;
        uint32_t ib = n_birds, io = n_occ;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t yb = __shfl_up_sync(FULL, ib, o), yo = __shfl_up_sync(FULL, io, o);
            if ((int)lane >= o) {
                ib += yb;
                io += yo;
            }
        }
        const int f = find_flock_b(fl, nfl, i0);
        uint32_t base = 0, obase = 0;
        if (lane == 31) {
            base = atomicAdd(&fl[f].cursor, ib);
            obase = atomicAdd(occ_count, io);
        }
        uint32_t run = __shfl_sync(FULL, base, 31) + __ldg(&fl[f].vbase) + ib - n_birds;
        uint32_t slot = __shfl_sync(FULL, obase, 31) + io - n_occ;
        const uint32_t cc[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (cc[k]) {
                offsets[b0 + k] = run;
                occ[slot++] = b0 + k;
                run += cc[k];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// pass 3: scatter by arrival rank
// ---------------------------------------------------------------------------
// Each bird's sort key goes to its slot in its bucket's run:
// slab << 62 | bird << 31 | (view index - vbase). Sorting it orders a run by
// z-slab, then bird index (bird index alone in grid-reporting steps, whose
// slabs are all 0). Bird and local view index are below 2^31.
__global__ void __launch_bounds__(256) k_scatter(const FlockDesc* __restrict__ fl, int nfl, uint32_t V, Arena ar,
                                                 const uint32_t* __restrict__ key, const uint32_t* __restrict__ arrival,
                                                 const uint32_t* __restrict__ offsets,
                                                 unsigned long long* __restrict__ tmp, StepCtl* __restrict__ ctl) {
    // two birds per thread and iteration (v and v + stride), so each thread has
    // two independent load chains in flight
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t v0 = blockIdx.x * blockDim.x + threadIdx.x; v0 < V; v0 += 2 * stride) {
        uint32_t bird[2], arr[2], kk[2], vb[2];
        bool act[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const uint32_t v = v0 + u * stride;
            act[u] = false;
            if (v < V) {
                const FlockDesc* d = &fl[find_flock_v(fl, nfl, v)];
                if (__ldg(&d->remaining)) {
                    act[u] = true;
                    vb[u] = __ldg(&d->vbase);
                    bird[u] = ar.id[v + view_shift(__ldg(&d->sbase), vb[u], __ldg(&d->parity), ar.cap)];
                    arr[u] = arrival[v];
                    kk[u] = key[v];
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            if (!act[u]) continue;
            const uint32_t v = v0 + u * stride;
            const uint32_t pos = __ldg(&offsets[kk[u]]) + (arr[u] & 0x3FFFFFFFu);
            if (pos < V)
                tmp[pos] = ((unsigned long long)(arr[u] >> 30) << 62) | ((unsigned long long)bird[u] << 31) |
                           (unsigned long long)(v - vb[u]);
            else atomicCAS(&ctl->error, 0u, (uint32_t)DEV_BAD_RANGE);
        }
    }
}

// ---------------------------------------------------------------------------
// pass 4: per-bucket stable order; state moves into cell order
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T kmin(T a, T b) { return a < b ? a : b; }
template <class T>
__device__ __forceinline__ T kmax(T a, T b) { return a < b ? b : a; }

template <class T>
__device__ __forceinline__ T bitonic32(T x, uint32_t lane) {
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            const T y = __shfl_xor_sync(FULL, x, j);
            const bool up = (lane & k) == 0;
            const bool lower = (lane & j) == 0;
            x = (lower == up) ? kmin(x, y) : kmax(x, y);
        }
    }
    return x;
}

// Bitonic sort of 32*R keys held R per lane (element i = lane + 32*k in x[k]),
// ascending; stages with stride >= 32 swap between a lane's own registers.
template <int R, class T>
__device__ __forceinline__ void bitonic_lanes(T (&x)[R], uint32_t lane) {
    constexpr int N = 32 * R;
#pragma unroll
    for (int s = 2; s <= N; s <<= 1) {
#pragma unroll
        for (int j = s >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
                const int jr = j >> 5;
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    const int kp = k ^ jr;
                    if (kp > k) {  // x[k] is the lower element of the pair
                        const bool up = ((lane + 32u * k) & (uint32_t)s) == 0;
                        const T a = x[k], b = x[kp];
                        x[k] = up ? kmin(a, b) : kmax(a, b);
                        x[kp] = up ? kmax(a, b) : kmin(a, b);
                    }
                }
            } else {
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    const uint32_t i = lane + 32u * k;
                    const T y = __shfl_xor_sync(FULL, x[k], j);
                    const bool up = (i & (uint32_t)s) == 0;
                    const bool lower = (i & (uint32_t)j) == 0;
                    x[k] = (lower == up) ? kmin(x[k], y) : kmax(x[k], y);
                }
            }
        }
    }
}

// A warp's deciding-bird records wait in shared memory and reach the global
// list in batches, one atomic on the list's counter per batch instead of one
// per bucket (that single counter was hit ~30,000 times per step at 1M birds).
constexpr uint32_t DUE_STAGE = 64;  // records per warp; flushed once more than 32 wait
constexpr uint32_t DUE_WORDS = sizeof(DueRec) / 16;  // 16-byte words per record

struct DueStage {
    DueRec* rec;   // this warp's DUE_STAGE records in shared memory
    uint32_t n;    // records waiting (warp-uniform)
};

// Adds the lanes' birds in slabs 0, 0-1 and 0-2 to c1, c2, c3 (warp-uniform).
__device__ __forceinline__ void slab_counts(bool has, unsigned long long x, uint32_t& c1, uint32_t& c2,
                                            uint32_t& c3) {
    const uint32_t sl = (uint32_t)(x >> 62);
    c1 += __popc(__ballot_sync(FULL, has && sl < 1u));
    c2 += __popc(__ballot_sync(FULL, has && sl < 2u));
    c3 += __popc(__ballot_sync(FULL, has && sl < 3u));
}

__device__ __forceinline__ void flush_due(DueStage& sg, uint32_t lane, DueRec* __restrict__ due,
                                          StepCtl* __restrict__ ctl) {
    if (!sg.n) return;
    __syncwarp();
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(&ctl->due_count, sg.n);
    base = __shfl_sync(FULL, base, 0);
    const uint4* src = reinterpret_cast<const uint4*>(sg.rec);
    uint4* dst = reinterpret_cast<uint4*>(due + base);
    for (uint32_t i = lane; i < sg.n * DUE_WORDS; i += 32) dst[i] = src[i];
    __syncwarp();
    sg.n = 0;
}

// Moves one bird (sort key x = slab << 62 | bird << 31 | old local view index) to view index
// `pos` of the reordered buffer, writes its unit heading to the forward view
// and, when it decides this step, stages its self-contained decide record.
// Called by all 32 lanes.
__device__ __forceinline__ void emit_sorted(bool has, uint32_t pos, unsigned long long x, const FlockDesc& d,
                                            float t_now, uint32_t lane, const Arena& ar, uint32_t oshift,
                                            uint32_t nshift, float4* __restrict__ sfwd, DueStage& sg,
                                            DueRec* __restrict__ due, StepCtl* __restrict__ ctl) {
    bool is_due = false;
    uint32_t nst = 0;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), c = a;
    f3 fw = mk(0.f, 0.f, 0.f);
    if (has && ((uint32_t)x & 0x7FFFFFFFu) >= d.n) {  // never with a consistent grid
        atomicCAS(&ctl->error, 0u, (uint32_t)DEV_BAD_RANGE);
        has = false;
    }
    if (has) {
        const uint32_t bird = (uint32_t)(x >> 31) & 0x7FFFFFFFu;
        const uint32_t ost = d.vbase + ((uint32_t)x & 0x7FFFFFFFu) + oshift;
        nst = pos + nshift;
        a = ar.A[ost];
        const float4 b = ar.B[ost];
        c = ar.C[ost];
        const float4 e = ar.D[ost];
        ar.A[nst] = a;
        ar.B[nst] = b;
        ar.C[nst] = c;
        ar.D[nst] = e;
        ar.id[nst] = bird;
        fw = forward(xyz(b));
        sfwd[pos] = make_float4(fw.x, fw.y, fw.z, 0.f);
        is_due = t_now >= e.x;
    }
    const uint32_t dm = __ballot_sync(FULL, is_due);
    if (dm) {
        if (is_due) {
            DueRec r;
            r.pr = make_float4(a.x, a.y, a.z, c.w);
            r.fk = make_float4(fw.x, fw.y, fw.z, __uint_as_float(pos));
            r.fl = make_uint4(nst, d.bbase, d.buckets, nshift);
            sg.rec[sg.n + __popc(dm & lanemask_lt())] = r;
        }
        sg.n += __popc(dm);
        if (sg.n > DUE_STAGE - 32) flush_due(sg, lane, due, ctl);
    }
}

// The pass waits on its loads. Each warp loads the bucket descriptors of 32
// buckets at once (one per lane: bucket, run start, length, flock), and the
// first 32 keys of the next run while the current one sorts (the 256-flock
// batch's sort 0.42 -> 0.39 ms, 64 registers, four CTAs per SM).
__global__ void __launch_bounds__(256, 4) k_segsort(const FlockDesc* __restrict__ fl, int nfl, uint32_t V,
                                                 StepCtl* __restrict__ ctl,
                                                 const uint32_t* __restrict__ occ, const uint32_t* __restrict__ offsets,
                                                 const uint32_t* __restrict__ counts,
                                                 const uint32_t* __restrict__ occ_count,
                                                 const unsigned long long* __restrict__ tmp, Arena ar,
                                                 float4* __restrict__ sfwd, DueRec* __restrict__ due,
                                                 uint32_t* __restrict__ slabs) {
    constexpr unsigned long long PAD = ~0ull;
    __shared__ DueRec s_due[8][DUE_STAGE];  // 256-thread CTAs: 8 warps
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t nocc = *(volatile const uint32_t*)occ_count;
    DueStage sg{s_due[(threadIdx.x >> 5) & 7], 0u};
    // each warp takes a contiguous range of occupied buckets (neighbouring
    // cells), so a batch of staged records stays spatially close for decide
    const uint32_t per = (nocc + nw - 1) / nw;
    const uint32_t w_beg = min(nocc, gw * per), w_end = min(nocc, w_beg + per);
    for (uint32_t c0 = w_beg; c0 < w_end; c0 += 32) {
        // the chunk's buckets, starts, lengths and flocks, one per lane, all loads in flight together
        const uint32_t cnt = min(32u, w_end - c0);
        uint32_t bl = 0, sl = 0, Ll = 0;
        int fl_ = 0;
        if (lane < cnt) {
            bl = occ[c0 + lane];
            sl = __ldg(&offsets[bl]);
            Ll = __ldg(&counts[bl]);
            fl_ = find_flock_b(fl, nfl, bl);
        }
        // the first 32 keys of the next bucket are loaded while this one is sorted
        auto first_keys = [&](uint32_t j) -> unsigned long long {
            const uint32_t s = __shfl_sync(FULL, sl, j), l = __shfl_sync(FULL, Ll, j);
            return (lane < l && s + l >= s && s + l <= V) ? tmp[s + lane] : PAD;
        };
        unsigned long long xn = first_keys(0);
        for (uint32_t j = 0; j < cnt; ++j) {
            const uint32_t b = __shfl_sync(FULL, bl, j);
            const int f = __shfl_sync(FULL, fl_, j);
            const uint32_t s0 = __shfl_sync(FULL, sl, j), L = __shfl_sync(FULL, Ll, j);
            const unsigned long long x0 = xn;
            if (j + 1 < cnt) xn = first_keys(j + 1);
            const FlockDesc d = fl[f];
            const float t_now = __fadd_rn(d.time, DT);
            const uint32_t oshift = view_shift(d.sbase, d.vbase, d.parity, ar.cap), nshift = view_shift(d.sbase, d.vbase, d.parity ^ 1u, ar.cap);
            // a run lies inside its flock's view region; never otherwise with valid
            // starts, and skipping keeps every slot inside the flock's own range
            if (s0 < d.vbase || s0 + L > d.vbase + d.n || s0 + L < s0 || s0 + L > V) {
                if (lane == 0) atomicCAS(&ctl->error, 0u, (uint32_t)DEV_BAD_RANGE);
                continue;
            }
            uint32_t c1 = 0, c2 = 0, c3 = 0;
            if (L <= 32) {
                unsigned long long x = x0;
                // runs often arrive in order already (birds are counted in the previous
                // step's cell order, a warp's birds with consecutive ranks)
                const unsigned long long nx = __shfl_down_sync(FULL, x, 1);
                const uint32_t dm = __ballot_sync(FULL, lane + 1 < L && x > nx);  // descents
                if (dm && (dm & (dm - 1))) {
                    x = bitonic32(x, lane);
                } else if (dm) {
                    // two ascending runs, lanes [0, k) and [k, L): with the second reversed
                    // into the top lanes and padding between, the 32 keys form a bitonic
                    // sequence, which one merge cascade sorts
                    const uint32_t k = (uint32_t)__ffs(dm), lb = L - k;
                    const uint32_t src = k + 31u - lane;  // lanes >= 32 - lb take B reversed
                    const unsigned long long y = __shfl_sync(FULL, x, src & 31u);
                    x = lane < k ? x : (lane >= 32u - lb ? y : PAD);
#pragma unroll
                    for (int j = 16; j > 0; j >>= 1) {
                        const unsigned long long z = __shfl_xor_sync(FULL, x, j);
                        x = (lane & (uint32_t)j) ? kmax(x, z) : kmin(x, z);
                    }
                }
                slab_counts(lane < L, x, c1, c2, c3);
                emit_sorted(lane < L, s0 + lane, x, d, t_now, lane, ar, oshift, nshift, sfwd, sg, due, ctl);
            } else if (L <= 64) {  // two cells in one bucket, or a dense cell: sort in registers
                unsigned long long x[2];
                x[0] = x0;
                x[1] = lane + 32u < L ? tmp[s0 + lane + 32u] : PAD;
                {
                    const unsigned long long n0 = __shfl_down_sync(FULL, x[0], 1);
                    const unsigned long long h1 = __shfl_sync(FULL, x[1], 0);
                    const unsigned long long n1 = __shfl_down_sync(FULL, x[1], 1);
                    const bool ok0 = lane < 31 ? x[0] < n0 : x[0] < h1;
                    const bool ok1 = lane + 33u >= L || x[1] < n1;
                    if (!__all_sync(FULL, ok0 && ok1)) bitonic_lanes<2>(x, lane);
                }
#pragma unroll
                for (int k = 0; k < 2; ++k)
                    slab_counts(lane + 32u * k < L, x[k], c1, c2, c3);
#pragma unroll
                for (int k = 0; k < 2; ++k)
                    emit_sorted(lane + 32u * k < L, s0 + lane + 32u * k, x[k], d, t_now, lane, ar, oshift, nshift, sfwd, sg,
                                due, ctl);
            } else if (L <= 128) {
                unsigned long long x[4];
#pragma unroll
                for (int k = 1; k < 4; ++k) x[k] = lane + 32u * k < L ? tmp[s0 + lane + 32u * k] : PAD;
                x[0] = x0;
                bitonic_lanes<4>(x, lane);
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    slab_counts(lane + 32u * k < L, x[k], c1, c2, c3);
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    emit_sorted(lane + 32u * k < L, s0 + lane + 32u * k, x[k], d, t_now, lane, ar, oshift, nshift, sfwd, sg,
                                due, ctl);
            } else {
                // long range (dense cell or hash collision): rank by counting; bird
                // indices are distinct within a flock, so ranks are distinct
                for (uint32_t k0 = 0; k0 < L; k0 += 32) {
                    const bool has = k0 + lane < L;
                    const unsigned long long x = has ? tmp[s0 + k0 + lane] : PAD;
                    uint32_t rank = 0;
                    for (uint32_t j0 = 0; j0 < L; j0 += 32) {
                        const unsigned long long y = (j0 + lane < L) ? tmp[s0 + j0 + lane] : PAD;
#pragma unroll 8
                        for (int q = 0; q < 32; ++q) rank += __shfl_sync(FULL, y, q) < x;
                    }
                    slab_counts(has, x, c1, c2, c3);
                    emit_sorted(has, s0 + rank, x, d, t_now, lane, ar, oshift, nshift, sfwd, sg, due, ctl);
                }
            }
            // the run's slab boundaries for decide (runs above 1023 birds are not trimmed)
            if (lane == 0) slabs[b] = L <= 1023u ? (c1 | (c2 << 10) | (c3 << 20)) : 0xFFFFFFFFu;
        }
    }
    // The CTA's remaining records go out in warp order, i.e. in the order of
    // its consecutive buckets, with one atomic: decide's warps take records in
    // list order, so each decide CTA works on one compact patch of cells.
    __shared__ uint32_t s_n[8], s_base;
    const uint32_t warp = (threadIdx.x >> 5) & 7;
    if (lane == 0) s_n[warp] = sg.n;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int k = 0; k < 8; ++k) t += s_n[k];
        s_base = t ? atomicAdd(&ctl->due_count, t) : 0u;
    }
    __syncthreads();
    uint32_t pre = s_base;
    for (uint32_t k = 0; k < warp; ++k) pre += s_n[k];
    const uint4* src = reinterpret_cast<const uint4*>(sg.rec);
    uint4* dst = reinterpret_cast<uint4*>(due + pre);
    for (uint32_t i = lane; i < sg.n * DUE_WORDS; i += 32) dst[i] = src[i];
}

}  // namespace flk
