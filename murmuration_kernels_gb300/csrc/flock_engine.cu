// GB300 (sm_103a) kernels and host engine for the starling-flock step.
//
// One step (reference order, crates/flock-ref/src/model.rs:182-200 and
// cuda/flock.cu:453-470): time += DT; rebuild the cell grid from the current
// positions; every bird with time >= next_decision decides from a snapshot;
// every bird integrates. The passes here:
//
//   k_hash_count  cell key per bird + bucket histogram with warp-aggregated
//                 atomics (__match_any_sync); records each bird's arrival rank
//                 and appends first-seen buckets to an occupied-bucket list.
//   k_scan        single-pass decoupled look-back exclusive scan of the
//                 histogram into bucket offsets (buckets+1 entries); it also
//                 zeroes the histogram for the next step. Bounded waits.
//   k_scatter     bird -> slot in its bucket's range (arrival order).
//   k_segsort     one warp per occupied bucket sorts its range by bird index
//                 (the canonical stable order), writes the cell-ordered float4
//                 view (pos+id, forward direction) and the deciding-bird list.
//   k_decide      one warp per deciding bird: the 2R neighbourhood's buckets
//                 are deduplicated with __match_any_sync, lanes sweep each
//                 bucket's contiguous float4 range, and warp shuffles reduce.
//   k_integrate   banked flight, streaming float4; its last block advances the
//                 flock clocks and resets the step counters.
//
// Exactness: the file is compiled with -fmad=false, and the expressions that
// decide set membership use explicit round-to-nearest intrinsics, so cell
// keys, the sorted order and all four neighbour sets equal the CPU oracle's
// bit for bit. Sums run in lane order instead of bird order, so forces agree
// to rounding (about 1e-7 relative), not bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "flock_engine.h"
#include "flock_params.h"

namespace flk {

#define FLK_CUDA(call)                                                                                    \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) {                                                                          \
            throw Error{-3, std::string(#call) + ": " + cudaGetErrorString(e_)};                          \
        }                                                                                                 \
    } while (0)

constexpr uint32_t FULL = 0xFFFFFFFFu;
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr uint32_t SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;  // 4096 buckets per tile
constexpr uint32_t SCAN_SPIN_LIMIT = 1u << 22;             // look-back polls before giving up
constexpr uint32_t FLAG_A = 1u, FLAG_P = 2u;

uint32_t buckets_for(uint32_t n) {
    uint64_t want = 1;
    while (want < (uint64_t)n * 2) want <<= 1;
    return (uint32_t)std::min<uint64_t>(std::max<uint64_t>(want, 1u << 16), 1u << 22);
}

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 add(f3 a, f3 b) { return mk(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)); }
__device__ __forceinline__ f3 sub(f3 a, f3 b) { return mk(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
__device__ __forceinline__ f3 mul(f3 a, float s) { return mk(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)); }
__device__ __forceinline__ f3 dvs(f3 a, float s) { return mk(__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s)); }
__device__ __forceinline__ float dot(f3 a, f3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
// glam Vec3::cross
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return mk(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(b.y, a.z)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(b.z, a.x)),
              __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(b.x, a.y)));
}
__device__ __forceinline__ float len(f3 a) { return __fsqrt_rn(dot(a, a)); }
__device__ __forceinline__ f3 normalize(f3 a) { return mul(a, __fdiv_rn(1.0f, len(a))); }
__device__ __forceinline__ f3 normalize_or_zero(f3 a) {
    const float rcp = __fdiv_rn(1.0f, len(a));
    return (isfinite(rcp) && rcp > 0.0f) ? mul(a, rcp) : mk(0.f, 0.f, 0.f);
}
// f32::clamp (NaN passes through)
__device__ __forceinline__ float clampf(float v, float lo, float hi) {
    if (v < lo) v = lo;
    if (v > hi) v = hi;
    return v;
}
// model.rs:15-38
__device__ __forceinline__ f3 forward(f3 v) { return dot(v, v) > 1e-12f ? normalize(v) : mk(1.f, 0.f, 0.f); }
__device__ __forceinline__ f3 side_of(f3 f) {
    const f3 s = cross(f, mk(0.f, 0.f, 1.f));
    return dot(s, s) > 1e-8f ? normalize(s) : mk(1.f, 0.f, 0.f);
}
__device__ __forceinline__ f3 body_up(f3 f, float beta) {
    const f3 side = side_of(f);
    const f3 up0 = cross(side, f);
    return add(mul(up0, cosf(beta)), mul(side, sinf(beta)));
}
__device__ __forceinline__ f3 xyz(float4 v) { return mk(v.x, v.y, v.z); }

// cuda/flock.cu:77-83: cell = floor(p / 4), bucket = spatial hash & mask.
__device__ __forceinline__ int cell1(float x) { return (int)floorf(__fmul_rn(x, INV_CELL)); }
__device__ __forceinline__ uint32_t cell_hash(int cx, int cy, int cz) {
    return ((uint32_t)cx * 73856093u) ^ ((uint32_t)cy * 19349663u) ^ ((uint32_t)cz * 83492791u);
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ int find_flock_v(const FlockDesc* __restrict__ fl, int nfl, uint32_t v) {
    int lo = 0, hi = nfl - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&fl[mid].vbase) <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int find_flock_b(const FlockDesc* __restrict__ fl, int nfl, uint32_t b) {
    int lo = 0, hi = nfl - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&fl[mid].bbase) <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// ---------------------------------------------------------------------------
// .flk words <-> arena (A = pos,roll  B = vel,spin  C = steer,radius  D = next,nb,cen)
// ---------------------------------------------------------------------------
__global__ void k_unpack(const float* __restrict__ w, uint32_t n, uint32_t sbase, float4* A, float4* B, float4* C,
                         float4* D) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* r = w + (size_t)i * WORDS;
        const uint32_t s = sbase + i;
        A[s] = make_float4(r[0], r[1], r[2], r[6]);
        B[s] = make_float4(r[3], r[4], r[5], r[7]);
        C[s] = make_float4(r[9], r[10], r[11], r[8]);
        D[s] = make_float4(r[12], r[13], r[14], 0.f);
    }
}

__global__ void k_pack(float* __restrict__ w, uint32_t n, uint32_t sbase, const float4* A, const float4* B,
                       const float4* C, const float4* D) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float* r = w + (size_t)i * WORDS;
        const uint32_t s = sbase + i;
        const float4 a = A[s], b = B[s], c = C[s], d = D[s];
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
__global__ void __launch_bounds__(256) k_hash_count(const FlockDesc* __restrict__ fl, int nfl, uint32_t V,
                                                    const float4* __restrict__ A, uint32_t* __restrict__ key,
                                                    uint32_t* __restrict__ arrival, uint32_t* __restrict__ counts,
                                                    uint32_t* __restrict__ occ, StepCtl* __restrict__ ctl) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t v0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); v0 < V; v0 += stride) {
        const uint32_t v = v0 + lane;
        bool act = false;
        uint32_t b = 0;
        if (v < V) {
            const FlockDesc* d = &fl[find_flock_v(fl, nfl, v)];
            if (__ldg(&d->remaining)) {
                const float4 p = A[__ldg(&d->sbase) + (v - __ldg(&d->vbase))];
                b = __ldg(&d->bbase) + (cell_hash(cell1(p.x), cell1(p.y), cell1(p.z)) & (__ldg(&d->buckets) - 1u));
                key[v] = b;
                act = true;
            }
        }
        const uint32_t m = __ballot_sync(FULL, act);
        if (act) {
            const uint32_t peers = __match_any_sync(m, b);
            const int leader = __ffs(peers) - 1;
            uint32_t old = 0;
            if ((int)lane == leader) old = atomicAdd(&counts[b], (uint32_t)__popc(peers));
            old = __shfl_sync(m, old, leader);
            const uint32_t rank = old + __popc(peers & lanemask_lt());
            arrival[v] = rank;
            const bool first = rank == 0;
            const uint32_t fm = __ballot_sync(m, first);
            if (fm) {
                const int wl = __ffs(m) - 1;
                uint32_t base = 0;
                if ((int)lane == wl) base = atomicAdd(&ctl->occ_count, (uint32_t)__popc(fm));
                base = __shfl_sync(m, base, wl);
                if (first) occ[base + __popc(fm & lanemask_lt())] = b;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// pass 2: single-pass decoupled look-back exclusive scan (counts -> offsets)
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long scan_word(uint32_t epoch, uint32_t flag, uint32_t value) {
    return ((unsigned long long)(epoch & 0x3FFFFFFFu) << 34) | ((unsigned long long)flag << 32) | value;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan(uint32_t* __restrict__ counts, uint32_t* __restrict__ offsets,
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

    uint4 c[SCAN_ITEMS / 4];
    uint4* src = reinterpret_cast<uint4*>(counts + base);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS / 4; ++k) c[k] = src[k];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS / 4; ++k) src[k] = make_uint4(0, 0, 0, 0);  // histogram ready for next step
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
            if (lane == 0) st_relaxed(&status[0], scan_word(epoch, FLAG_P, agg));
        } else {
            if (lane == 0) st_relaxed(&status[tile], scan_word(epoch, FLAG_A, agg));
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
                    if (++polls > SCAN_SPIN_LIMIT) {  // give up: record and let every waiter finish
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
            if (lane == 0) st_relaxed(&status[tile], scan_word(epoch, FLAG_P, excl + agg));
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
// pass 3: scatter by arrival rank
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_scatter(const FlockDesc* __restrict__ fl, int nfl, uint32_t V,
                                                 const uint32_t* __restrict__ key, const uint32_t* __restrict__ arrival,
                                                 const uint32_t* __restrict__ offsets, uint32_t* __restrict__ tmp,
                                                 StepCtl* __restrict__ ctl) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        const FlockDesc* d = &fl[find_flock_v(fl, nfl, v)];
        if (!__ldg(&d->remaining)) continue;
        const uint32_t pos = __ldg(&offsets[key[v]]) + arrival[v];
        if (pos < V) tmp[pos] = v;
        else atomicCAS(&ctl->error, 0u, (uint32_t)DEV_BAD_RANGE);
    }
}

// ---------------------------------------------------------------------------
// pass 4: per-bucket stable order + cell-ordered view + deciding-bird list
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t bitonic32(uint32_t x, uint32_t lane) {
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            const uint32_t y = __shfl_xor_sync(FULL, x, j);
            const bool up = (lane & k) == 0;
            const bool lower = (lane & j) == 0;
            x = (lower == up) ? min(x, y) : max(x, y);
        }
    }
    return x;
}

__device__ __forceinline__ void emit_sorted(bool has, uint32_t pos, uint32_t v, const FlockDesc& d, int f, float t_now,
                                            uint32_t lane, const float4* __restrict__ A, const float4* __restrict__ B,
                                            const float4* __restrict__ D, uint32_t* __restrict__ sorted,
                                            float4* __restrict__ spos, float4* __restrict__ sfwd,
                                            uint2* __restrict__ due, StepCtl* __restrict__ ctl) {
    bool is_due = false;
    if (has) {
        const uint32_t local = v - d.vbase;
        const uint32_t st = d.sbase + local;
        const float4 a = A[st];
        const float4 b = B[st];
        const float nd = __ldg(&D[st].x);
        sorted[pos] = local;
        spos[pos] = make_float4(a.x, a.y, a.z, __uint_as_float(local));
        const f3 fw = forward(xyz(b));
        sfwd[pos] = make_float4(fw.x, fw.y, fw.z, 0.f);
        is_due = t_now >= nd;
    }
    const uint32_t dm = __ballot_sync(FULL, is_due);
    if (dm) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&ctl->due_count, (uint32_t)__popc(dm));
        base = __shfl_sync(FULL, base, 0);
        if (is_due) due[base + __popc(dm & lanemask_lt())] = make_uint2(pos, (uint32_t)f);
    }
}

__global__ void __launch_bounds__(256) k_segsort(const FlockDesc* __restrict__ fl, int nfl, uint32_t V,
                                                 StepCtl* __restrict__ ctl,
                                                 const uint32_t* __restrict__ occ, const uint32_t* __restrict__ offsets,
                                                 const uint32_t* __restrict__ tmp, const float4* __restrict__ A,
                                                 const float4* __restrict__ B, const float4* __restrict__ D,
                                                 uint32_t* __restrict__ sorted, float4* __restrict__ spos,
                                                 float4* __restrict__ sfwd, uint2* __restrict__ due) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t nocc = *(volatile uint32_t*)&ctl->occ_count;
    for (uint32_t w = gw; w < nocc; w += nw) {
        const uint32_t b = occ[w];
        const int f = find_flock_b(fl, nfl, b);
        const FlockDesc d = fl[f];
        const float t_now = __fadd_rn(d.time, DT);
        const uint32_t s0 = __ldg(&offsets[b]), e0 = __ldg(&offsets[b + 1]);
        if (e0 < s0 || e0 > V) {  // never with a completed scan; skip rather than read out of range
            if (lane == 0) atomicCAS(&ctl->error, 0u, (uint32_t)DEV_BAD_RANGE);
            continue;
        }
        const uint32_t L = e0 - s0;
        if (L <= 32) {
            uint32_t x = lane < L ? tmp[s0 + lane] : 0xFFFFFFFFu;
            x = bitonic32(x, lane);
            emit_sorted(lane < L, s0 + lane, x, d, f, t_now, lane, A, B, D, sorted, spos, sfwd, due, ctl);
        } else {
            // long range (dense cell or hash collision): rank by counting
            for (uint32_t c0 = 0; c0 < L; c0 += 32) {
                const bool has = c0 + lane < L;
                const uint32_t x = has ? tmp[s0 + c0 + lane] : 0xFFFFFFFFu;
                uint32_t rank = 0;
                for (uint32_t j0 = 0; j0 < L; j0 += 32) {
                    const uint32_t y = (j0 + lane < L) ? tmp[s0 + j0 + lane] : 0xFFFFFFFFu;
#pragma unroll 8
                    for (int q = 0; q < 32; ++q) rank += __shfl_sync(FULL, y, q) < x;
                }
                emit_sorted(has, s0 + rank, x, d, f, t_now, lane, A, B, D, sorted, spos, sfwd, due, ctl);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// pass 5: decide (model.rs:53-145), one warp per deciding bird
// ---------------------------------------------------------------------------
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

// One candidate. CHECK_CELL: only birds of cell (cx,cy,cz) count (the cell
// walk, where one bucket can be visited for several cells).
template <bool SETS, bool CHECK_CELL>
__device__ __forceinline__ void visit(uint32_t t, uint32_t self, f3 p, f3 fi, float r2, float c2,
                                      const float4* __restrict__ spos, const float4* __restrict__ sfwd, Acc& a, int cx = 0,
                                      int cy = 0, int cz = 0) {
    if (t == self) return;
    const float4 q = __ldg(&spos[t]);
    if (CHECK_CELL) {
        if (cell1(q.x) != cx || cell1(q.y) != cy || cell1(q.z) != cz) return;
    }
    const f3 d = mk(__fsub_rn(q.x, p.x), __fsub_rn(q.y, p.y), __fsub_rn(q.z, p.z));
    const float d2 = dot(d, d);
    if (d2 > c2) return;
    const float dist = __fsqrt_rn(d2);
    const f3 dh = dvs(d, fmaxf(dist, 1e-6f));
    a.csum = add(a.csum, dh);
    a.n_g += 1;
    const uint32_t j = __float_as_uint(q.w);
    if (SETS) a.h_g += set_mix(j);
    if (d2 > r2) return;
    a.n_all += 1;
    if (SETS) a.h_all += set_mix(j);
    float g = 1.0f;
    if (dist > R_H) {
        const float tt = __fsub_rn(dist, R_H);
        g = expf(__fdiv_rn(-__fmul_rn(tt, tt), TWO_SIGMA2));
    }
    a.sep = sub(a.sep, mul(dh, g));
    if (dist > R_H) {
        a.coh = add(a.coh, dh);
        a.n_star += 1;
        if (SETS) a.h_star += set_mix(j);
    }
    if (dot(fi, dh) >= BLIND_COS) {
        const float4 fw = __ldg(&sfwd[t]);
        a.align = add(a.align, xyz(fw));
        a.n_align += 1;
        if (SETS) a.h_align += set_mix(j);
    }
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

template <bool SETS>
__global__ void __launch_bounds__(256) k_decide(const FlockDesc* __restrict__ fl, uint32_t V, StepCtl* __restrict__ ctl,
                                                const uint2* __restrict__ due, const uint32_t* __restrict__ offsets,
                                                const float4* __restrict__ spos, const float4* __restrict__ sfwd,
                                                const float4* __restrict__ Bv, float4* __restrict__ C,
                                                float4* __restrict__ D, const float* __restrict__ rtab,
                                                uint32_t* __restrict__ sets) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t ndue = *(volatile uint32_t*)&ctl->due_count;
    unsigned long long cand = 0, pairs = 0;

    for (uint32_t e = gw; e < ndue; e += nw) {
        const uint2 ent = due[e];
        const uint32_t k = ent.x;
        const FlockDesc d = fl[ent.y];
        const float4 me = spos[k];
        const uint32_t local = __float_as_uint(me.w);
        const uint32_t st = d.sbase + local;
        const float4 cme = C[st];
        const float4 vme = Bv[st];
        const float r = cme.w;
        const f3 p = mk(me.x, me.y, me.z);
        const f3 v = xyz(vme);
        const f3 fi = forward(v);
        const float r2 = __fmul_rn(r, r);
        const float rr = __fmul_rn(2.0f, r);
        const float c2 = __fmul_rn(rr, rr);
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

        Acc a;
        a.sep = a.coh = a.align = a.csum = mk(0.f, 0.f, 0.f);
        a.n_all = a.n_star = a.n_align = a.n_g = 0;
        a.h_all = a.h_star = a.h_align = a.h_g = 0;

        if (ncell <= 32) {
            // fast path: visit each distinct bucket of the culled box once, no cell check
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
            uint32_t km = __ballot_sync(FULL, keep);
            uint32_t s = 0, en = 0;
            if (keep) bucket_range(offsets, b, V, ctl, s, en);
            while (km) {
                const int c = __ffs(km) - 1;
                km &= km - 1;
                const uint32_t sc = __shfl_sync(FULL, s, c), ec = __shfl_sync(FULL, en, c);
                cand += ec - sc;
                for (uint32_t t = sc + lane; t < ec; t += 32) visit<SETS, false>(t, k, p, fi, r2, c2, spos, sfwd, a);
            }
        } else {
            uint32_t f0 = __ldg(&offsets[d.bbase]), f1 = __ldg(&offsets[d.bbase + d.buckets]);
            if (f1 < f0 || f1 > V) f1 = f0 = 0;
            if (ncell * 16 >= (long long)(f1 - f0)) {
                // very wide reach: brute force over the flock's own range
                cand += f1 - f0;
                for (uint32_t t = f0 + lane; t < f1; t += 32) visit<SETS, false>(t, k, p, fi, r2, c2, spos, sfwd, a);
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
                            const uint32_t b = d.bbase + (cell_hash(cx, cy, cz) & mask);
                            bucket_range(offsets, b, V, ctl, s, en);
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
                        for (uint32_t t = sc + lane; t < ec; t += 32)
                            visit<SETS, true>(t, k, p, fi, r2, c2, spos, sfwd, a, ccx, ccy, ccz);
                    }
                }
            }
        }

        // warp reduction (fixed butterfly; lane 0's association is deterministic)
        const f3 sep = wsum3(a.sep), coh = wsum3(a.coh), align = wsum3(a.align), csum = wsum3(a.csum);
        const uint32_t n_all = wsumu(a.n_all), n_star = wsumu(a.n_star), n_align = wsumu(a.n_align), n_g = wsumu(a.n_g);
        uint32_t h_all = 0, h_star = 0, h_align = 0, h_g = 0;
        if (SETS) {
            h_all = wsumu(a.h_all);
            h_star = wsumu(a.h_star);
            h_align = wsumu(a.h_align);
            h_g = wsumu(a.h_g);
        }
        if (lane == 0) {
            pairs += n_g;
            f3 force = mk(0.f, 0.f, 0.f);
            if (n_all > 0) force = add(force, mul(sep, __fdiv_rn(W_SEP, (float)n_all)));
            const float cen = n_g > 0 ? __fdiv_rn(len(csum), (float)n_g) : 0.0f;
            if (n_star > 0) force = add(force, mul(normalize_or_zero(coh), __fmul_rn(W_COH, cen)));
            const f3 al = n_align > 0 ? sub(dvs(align, (float)n_align), fi) : mk(0.f, 0.f, 0.f);
            force = add(force, mul(al, W_ALIGN));
            const float roost = __fmul_rn(W_ROOST_V, clampf(__fdiv_rn(__fsub_rn(Z0, p.z), H_ROOST_V), -1.0f, 1.0f));
            force = add(force, mul(mk(0.f, 0.f, 1.f), roost));
            const float speed = len(v);
            force = add(force, mul(fi, __fmul_rn(MASS / TAU, __fsub_rn(V0, speed))));
            const float nd = D[st].x;
            C[st] = make_float4(force.x, force.y, force.z, radius_step(r, n_all, rtab));
            D[st] = make_float4(__fadd_rn(nd, DU), __uint_as_float(n_all), cen, 0.f);
            if (SETS) {
                uint32_t* o = sets + (size_t)(d.vbase + local) * 8;
                o[0] = n_all; o[1] = n_star; o[2] = n_align; o[3] = n_g;
                o[4] = h_all; o[5] = h_star; o[6] = h_align; o[7] = h_g;
            }
        }
    }
    // per-block totals, one atomic per block
    __shared__ unsigned long long s_cand, s_pairs, s_due;
    if (threadIdx.x == 0) s_cand = s_pairs = s_due = 0;
    __syncthreads();
    if (lane == 0 && (cand | pairs)) {
        atomicAdd(&s_cand, cand);
        atomicAdd(&s_pairs, pairs);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_cand) atomicAdd(&ctl->cand_total, s_cand);
        if (s_pairs) atomicAdd(&ctl->pair_total, s_pairs);
        if (blockIdx.x == 0) atomicAdd(&ctl->due_total, (unsigned long long)ndue);
    }
}

// ---------------------------------------------------------------------------
// pass 6: integrate (model.rs:149-176) + end-of-step bookkeeping
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_integrate(FlockDesc* __restrict__ fl, int nfl, uint32_t V,
                                                   float4* __restrict__ A, float4* __restrict__ B,
                                                   const float4* __restrict__ C, StepCtl* __restrict__ ctl) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        const FlockDesc* d = &fl[find_flock_v(fl, nfl, v)];
        if (!d->remaining) continue;
        const uint32_t st = d->sbase + (v - d->vbase);
        const float4 a = A[st];
        const float4 b = B[st];
        const float4 c = C[st];
        f3 vel = xyz(b);
        const f3 steering = xyz(c);
        const float roll = a.w;

        const f3 fw = forward(vel);
        const f3 side = side_of(fw);
        const float speed = fmaxf(len(vel), 1e-6f);
        const float a_lat = __fdiv_rn(dot(steering, side), MASS);
        const float target = clampf(atanf(__fdiv_rn(a_lat, G)), -MAX_BANK, MAX_BANK);
        const float rate = clampf(__fdiv_rn(__fsub_rn(target, roll), TAU_ROLL), -MAX_ROLL_RATE, MAX_ROLL_RATE);
        const float beta = clampf(__fadd_rn(roll, __fmul_rn(rate, DT)), -MAX_BANK, MAX_BANK);

        const f3 up = body_up(fw, beta);
        const float cos_beta = fmaxf(cosf(beta), 0.2f);
        const float sr = __fdiv_rn(speed, V0);
        const float sr2 = __fmul_rn(sr, sr);
        const float lift = __fdiv_rn(__fmul_rn(sr2, L0), cos_beta);
        const float drag = __fmul_rn(sr2, D0);
        const f3 flight = sub(add(sub(mul(up, lift), mul(fw, drag)), mul(fw, D0)), mul(mul(mk(0.f, 0.f, 1.f), MASS), G));
        const f3 control = sub(steering, mul(side, dot(steering, side)));
        vel = add(vel, mul(dvs(add(control, flight), MASS), DT));
        const float sp = len(vel);
        if (sp > V_MAX) {
            vel = mul(vel, __fdiv_rn(V_MAX, sp));
        } else if (sp < V_MIN && sp > 1e-6f) {
            vel = mul(vel, __fdiv_rn(V_MIN, sp));
        }
        const f3 pos = add(xyz(a), mul(vel, DT));
        A[st] = make_float4(pos.x, pos.y, pos.z, beta);
        B[st] = make_float4(vel.x, vel.y, vel.z, rate);
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
            if (fl[f].remaining) {
                fl[f].time = __fadd_rn(fl[f].time, DT);
                fl[f].remaining -= 1;
            }
        }
        if (threadIdx.x == 0) {
            ctl->occ_count = 0;
            ctl->due_count = 0;
            ctl->scan_ticket = 0;
            ctl->epoch = ctl->epoch + 1;
            ctl->done_blocks = 0;
        }
    }
}

// ---------------------------------------------------------------------------
// host engine
// ---------------------------------------------------------------------------
template <class T>
static T* dalloc(size_t n, size_t* acct) {
    void* p = nullptr;
    if (n == 0) n = 1;
    FLK_CUDA(cudaMalloc(&p, n * sizeof(T)));
    *acct += n * sizeof(T);
    return static_cast<T*>(p);
}
template <class T>
static void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

Engine::Engine(int device) {
    if (device < 0) FLK_CUDA(cudaGetDevice(&device));
    device_ = device;
    FLK_CUDA(cudaSetDevice(device_));
    FLK_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, device_));
    FLK_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    ctl_ = dalloc<StepCtl>(1, &dev_bytes_);
    StepCtl c{};
    c.epoch = 1;
    FLK_CUDA(cudaMemcpyAsync(ctl_, &c, sizeof c, cudaMemcpyHostToDevice, stream_));
    std::vector<float> tab(RADIUS_TABLE);
    for (int n = 0; n < RADIUS_TABLE; ++n) {
        const float nn = (float)(n > 1 ? n : 1);
        tab[n] = powf(N_C / nn, RADIUS_EXP);
    }
    radius_table_ = dalloc<float>(RADIUS_TABLE, &dev_bytes_);
    FLK_CUDA(cudaMemcpyAsync(radius_table_, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, stream_));
    FLK_CUDA(cudaStreamSynchronize(stream_));
}

Engine::~Engine() {
    cudaSetDevice(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    free_graphs();
    dfree(A_); dfree(B_); dfree(C_); dfree(D_);
    dfree(table_d_);
    dfree(key_); dfree(arrival_); dfree(tmp_); dfree(sorted_); dfree(occ_); dfree(due_);
    dfree(spos_); dfree(sfwd_); dfree(counts_); dfree(offsets_); dfree(status_); dfree(sets_);
    dfree(ctl_); dfree(radius_table_); dfree(staging_);
    if (stream_) cudaStreamDestroy(stream_);
}

void Engine::free_graphs() {
    if (graph_) cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
    graph_steps_ = 0;
}

size_t Engine::bytes_for(uint32_t n) {
    // state 64 B + scratch (key, arrival, tmp, sorted, occ 4 B each; due 8 B;
    // spos, sfwd 16 B each) + buckets (counts 4 B + offsets 4 B + status/4096)
    const size_t b = buckets_for(n);
    return (size_t)n * (64 + 20 + 8 + 32) + b * 8 + (b / SCAN_TILE) * 8 + 256;
}

void Engine::set_shape(const LaunchShape& s) {
    shape_ = s;
    free_graphs();
}

void Engine::ensure_arena(uint32_t need) {
    if (need <= cap_) return;
    uint32_t ncap = std::max<uint32_t>(need, cap_ ? cap_ + cap_ / 2 : need);
    size_t acct = 0;
    float4 *a = dalloc<float4>(ncap, &acct), *b = dalloc<float4>(ncap, &acct), *c = dalloc<float4>(ncap, &acct),
           *d = dalloc<float4>(ncap, &acct);
    if (used_) {
        FLK_CUDA(cudaMemcpyAsync(a, A_, (size_t)used_ * 16, cudaMemcpyDeviceToDevice, stream_));
        FLK_CUDA(cudaMemcpyAsync(b, B_, (size_t)used_ * 16, cudaMemcpyDeviceToDevice, stream_));
        FLK_CUDA(cudaMemcpyAsync(c, C_, (size_t)used_ * 16, cudaMemcpyDeviceToDevice, stream_));
        FLK_CUDA(cudaMemcpyAsync(d, D_, (size_t)used_ * 16, cudaMemcpyDeviceToDevice, stream_));
        FLK_CUDA(cudaStreamSynchronize(stream_));
    }
    dev_bytes_ -= (size_t)cap_ * 64;
    dfree(A_); dfree(B_); dfree(C_); dfree(D_);
    A_ = a; B_ = b; C_ = c; D_ = d;
    dev_bytes_ += acct;
    cap_ = ncap;
    free_graphs();
}

int Engine::add_flock(uint32_t n, float time, const float* words) {
    FLK_CUDA(cudaSetDevice(device_));
    // first-fit into a hole, else append
    uint32_t sbase = used_;
    bool from_hole = false;
    for (auto& h : free_ranges_) {
        if (h.second >= n) {
            sbase = h.first;
            h.first += n;
            h.second -= n;
            from_hole = true;
            break;
        }
    }
    if (!from_hole) {
        ensure_arena(used_ + n);
        used_ += n;
    }
    free_ranges_.erase(std::remove_if(free_ranges_.begin(), free_ranges_.end(),
                                      [](const std::pair<uint32_t, uint32_t>& h) { return h.second == 0; }),
                       free_ranges_.end());
    if (n) {
        const size_t bytes = (size_t)n * WORDS * 4;
        if (bytes > staging_cap_) {
            dev_bytes_ -= staging_cap_;
            dfree(staging_);
            staging_ = dalloc<float>((size_t)n * WORDS, &dev_bytes_);
            staging_cap_ = bytes;
        }
        FLK_CUDA(cudaMemcpyAsync(staging_, words, bytes, cudaMemcpyHostToDevice, stream_));
        const int blocks = std::min<uint32_t>((n + 255) / 256, (uint32_t)num_sms_ * 8);
        k_unpack<<<blocks, 256, 0, stream_>>>(staging_, n, sbase, A_, B_, C_, D_);
        FLK_CUDA(cudaGetLastError());
    }
    Slot s;
    s.n = n;
    s.sbase = sbase;
    s.buckets = buckets_for(n);
    s.remaining = 0;
    s.time = time;
    s.live = true;
    int id = -1;
    for (size_t k = 0; k < slots_.size(); ++k)
        if (!slots_[k].live) { id = (int)k; break; }
    if (id < 0) {
        id = (int)slots_.size();
        slots_.push_back(s);
    } else {
        slots_[id] = s;
    }
    return id;
}

bool Engine::has_flock(int id) const { return id >= 0 && id < (int)slots_.size() && slots_[id].live; }
uint32_t Engine::flock_size(int id) const { return has_flock(id) ? slots_[id].n : 0; }
std::vector<int> Engine::flock_ids() const {
    std::vector<int> ids;
    for (size_t k = 0; k < slots_.size(); ++k)
        if (slots_[k].live) ids.push_back((int)k);
    return ids;
}

void Engine::sync_times() {
    // The device table holds the live clocks and countdowns once steps have
    // run; until then the host copy is authoritative (it may hold step counts
    // set since the last run that the device has not seen yet).
    if (!device_ahead_ || table_h_.empty() || !table_d_) return;
    device_ahead_ = false;
    std::vector<FlockDesc> t(table_h_.size());
    FLK_CUDA(cudaMemcpyAsync(t.data(), table_d_, t.size() * sizeof(FlockDesc), cudaMemcpyDeviceToHost, stream_));
    FLK_CUDA(cudaStreamSynchronize(stream_));
    for (size_t k = 0; k < t.size(); ++k) {
        if (table_ids_[k] < 0) continue;  // removed since the table was built
        Slot& s = slots_[table_ids_[k]];
        s.time = t[k].time;
        s.remaining = t[k].remaining;
    }
    table_h_ = t;
}

void Engine::remove_flock(int id) {
    if (!has_flock(id)) throw Error{-4, "unknown flock id"};
    sync_times();
    // the slot id may be reused before the table is rebuilt: detach it
    for (int& t : table_ids_)
        if (t == id) t = -1;
    Slot& s = slots_[id];
    s.live = false;
    if (s.n) {
        free_ranges_.push_back({s.sbase, s.n});
        std::sort(free_ranges_.begin(), free_ranges_.end());
        std::vector<std::pair<uint32_t, uint32_t>> merged;
        for (auto& h : free_ranges_) {
            if (!merged.empty() && merged.back().first + merged.back().second == h.first) merged.back().second += h.second;
            else merged.push_back(h);
        }
        // a hole at the end of the arena returns to the tail
        if (!merged.empty() && merged.back().first + merged.back().second == used_) {
            used_ = merged.back().first;
            merged.pop_back();
        }
        free_ranges_ = merged;
    }
    table_dirty_ = true;
}

float Engine::flock_time(int id) {
    if (!has_flock(id)) throw Error{-4, "unknown flock id"};
    sync_times();
    return slots_[id].time;
}

void Engine::read_flock(int id, float* time, float* words) {
    if (!has_flock(id)) throw Error{-4, "unknown flock id"};
    FLK_CUDA(cudaSetDevice(device_));
    sync_times();
    const Slot& s = slots_[id];
    if (time) *time = s.time;
    if (!s.n) return;
    const size_t bytes = (size_t)s.n * WORDS * 4;
    if (bytes > staging_cap_) {
        dev_bytes_ -= staging_cap_;
        dfree(staging_);
        staging_ = dalloc<float>((size_t)s.n * WORDS, &dev_bytes_);
        staging_cap_ = bytes;
    }
    const int blocks = std::min<uint32_t>((s.n + 255) / 256, (uint32_t)num_sms_ * 8);
    k_pack<<<blocks, 256, 0, stream_>>>(staging_, s.n, s.sbase, A_, B_, C_, D_);
    FLK_CUDA(cudaGetLastError());
    FLK_CUDA(cudaMemcpyAsync(words, staging_, bytes, cudaMemcpyDeviceToHost, stream_));
    FLK_CUDA(cudaStreamSynchronize(stream_));
}

void Engine::set_remaining(const std::vector<int>& ids, const std::vector<uint32_t>& steps) {
    sync_times();
    for (auto& s : slots_) s.remaining = 0;
    for (size_t k = 0; k < ids.size(); ++k) {
        if (!has_flock(ids[k])) throw Error{-4, "unknown flock id"};
        slots_[ids[k]].remaining = steps[k];
    }
    table_dirty_ = true;
}

void Engine::set_flock_remaining(int id, uint32_t steps) {
    if (!has_flock(id)) throw Error{-4, "unknown flock id"};
    sync_times();
    slots_[id].remaining = steps;
    table_dirty_ = true;
}

uint32_t Engine::flock_remaining(int id) {
    if (!has_flock(id)) throw Error{-4, "unknown flock id"};
    sync_times();
    return slots_[id].remaining;
}

std::vector<uint32_t> Engine::remaining_of(const std::vector<int>& ids) {
    sync_times();
    std::vector<uint32_t> out;
    for (int id : ids) {
        if (!has_flock(id)) throw Error{-4, "unknown flock id"};
        out.push_back(slots_[id].remaining);
    }
    return out;
}

double Engine::time_run(uint32_t steps) {
    FLK_CUDA(cudaSetDevice(device_));
    if (table_dirty_) {
        sync_times();
        rebuild_table();
    }
    cudaEvent_t e0, e1;
    FLK_CUDA(cudaEventCreate(&e0));
    FLK_CUDA(cudaEventCreate(&e1));
    // capture (if needed) before the timed region so the events bracket launches only
    if (!table_h_.empty() && steps >= (uint32_t)std::max(1, shape_.graph_chunk)) ensure_graph();
    FLK_CUDA(cudaEventRecord(e0, stream_));
    run(steps);
    FLK_CUDA(cudaEventRecord(e1, stream_));
    FLK_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    FLK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

__global__ void k_flush(uint4* __restrict__ buf, size_t n16, uint32_t salt) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
        buf[i] = make_uint4(salt, (uint32_t)i, salt, (uint32_t)i);
}

void Engine::time_steps_cold(uint32_t steps, size_t flush_bytes, float* ms_per_step) {
    FLK_CUDA(cudaSetDevice(device_));
    if (table_dirty_) {
        sync_times();
        rebuild_table();
    }
    if (table_h_.empty() || steps == 0) return;
    uint4* flush = nullptr;
    const size_t n16 = flush_bytes / 16;
    if (n16) FLK_CUDA(cudaMalloc(&flush, n16 * 16));
    cudaGraph_t g;
    cudaGraphExec_t one = nullptr;
    FLK_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    enqueue_step(false);
    FLK_CUDA(cudaStreamEndCapture(stream_, &g));
    cudaError_t e = cudaGraphInstantiate(&one, g, 0);
    cudaGraphDestroy(g);
    FLK_CUDA(e);
    std::vector<cudaEvent_t> ev(2 * (size_t)steps);
    for (auto& x : ev) FLK_CUDA(cudaEventCreate(&x));
    device_ahead_ = true;
    for (uint32_t s = 0; s < steps; ++s) {
        if (n16) k_flush<<<num_sms_ * 4, 256, 0, stream_>>>(flush, n16, s);
        FLK_CUDA(cudaEventRecord(ev[2 * s], stream_));
        FLK_CUDA(cudaGraphLaunch(one, stream_));
        FLK_CUDA(cudaEventRecord(ev[2 * s + 1], stream_));
    }
    FLK_CUDA(cudaGetLastError());
    FLK_CUDA(cudaStreamSynchronize(stream_));
    for (uint32_t s = 0; s < steps; ++s) FLK_CUDA(cudaEventElapsedTime(&ms_per_step[s], ev[2 * s], ev[2 * s + 1]));
    for (auto& x : ev) cudaEventDestroy(x);
    cudaGraphExecDestroy(one);
    if (flush) cudaFree(flush);
    for (size_t k = 0; k < table_h_.size(); ++k) {
        const uint32_t left = table_h_[k].remaining > steps ? table_h_[k].remaining - steps : 0;
        table_h_[k].remaining = left;
        if (table_ids_[k] >= 0) slots_[table_ids_[k]].remaining = left;
    }
    table_dirty_ = true;
}

void Engine::rebuild_table() {
    std::vector<FlockDesc> t;
    std::vector<int> ids;
    uint32_t V = 0;
    uint64_t Bt = 0;
    for (size_t k = 0; k < slots_.size(); ++k) {
        const Slot& s = slots_[k];
        if (!s.live || s.remaining == 0) continue;
        FlockDesc d{};
        d.vbase = V;
        d.n = s.n;
        d.sbase = s.sbase;
        d.bbase = (uint32_t)Bt;
        d.buckets = s.buckets;
        d.remaining = s.remaining;
        d.time = s.time;
        t.push_back(d);
        ids.push_back((int)k);
        V += s.n;
        Bt += s.buckets;
    }
    if (Bt >= (1ull << 32) - SCAN_TILE) throw Error{-5, "too many buckets in one batch"};
    if ((uint32_t)t.size() > table_cap_ || !table_d_) {
        dev_bytes_ -= (size_t)table_cap_ * sizeof(FlockDesc);
        dfree(table_d_);
        table_cap_ = std::max<uint32_t>((uint32_t)t.size(), 16);
        table_d_ = dalloc<FlockDesc>(table_cap_, &dev_bytes_);
    }
    if (!t.empty())
        FLK_CUDA(cudaMemcpyAsync(table_d_, t.data(), t.size() * sizeof(FlockDesc), cudaMemcpyHostToDevice, stream_));
    // a captured graph bakes in sizes and pointers, not the table contents
    const bool same_shape = t.size() == table_h_.size() && V == V_ && (uint32_t)Bt == Btot_;
    table_h_ = t;
    table_ids_ = ids;
    V_ = V;
    Btot_ = (uint32_t)Bt;
    if (!same_shape) free_graphs();
    ensure_scratch();
    table_dirty_ = false;
    device_ahead_ = false;  // the device table now equals the host copy
}

void Engine::ensure_scratch() {
    if (V_ > scratch_V_ || !key_) {
        const uint32_t nv = std::max<uint32_t>(V_, scratch_V_ + scratch_V_ / 2);
        dev_bytes_ -= (size_t)scratch_V_ * (20 + 8 + 32 + 32);
        dfree(key_); dfree(arrival_); dfree(tmp_); dfree(sorted_); dfree(occ_); dfree(due_);
        dfree(spos_); dfree(sfwd_); dfree(sets_);
        key_ = dalloc<uint32_t>(nv, &dev_bytes_);
        arrival_ = dalloc<uint32_t>(nv, &dev_bytes_);
        tmp_ = dalloc<uint32_t>(nv, &dev_bytes_);
        sorted_ = dalloc<uint32_t>(nv, &dev_bytes_);
        occ_ = dalloc<uint32_t>(nv, &dev_bytes_);
        due_ = dalloc<uint2>(nv, &dev_bytes_);
        spos_ = dalloc<float4>(nv, &dev_bytes_);
        sfwd_ = dalloc<float4>(nv, &dev_bytes_);
        scratch_V_ = nv;
        free_graphs();
    }
    if (Btot_ > scratch_B_) {
        const uint32_t nb = Btot_;
        dev_bytes_ -= (size_t)scratch_B_ * 8 + (scratch_B_ / SCAN_TILE) * 8;
        dfree(counts_); dfree(offsets_); dfree(status_);
        counts_ = dalloc<uint32_t>(nb, &dev_bytes_);
        offsets_ = dalloc<uint32_t>((size_t)nb + 1, &dev_bytes_);
        status_ = dalloc<unsigned long long>(nb / SCAN_TILE, &dev_bytes_);
        FLK_CUDA(cudaMemsetAsync(counts_, 0, (size_t)nb * 4, stream_));
        FLK_CUDA(cudaMemsetAsync(status_, 0, (size_t)(nb / SCAN_TILE) * 8, stream_));
        scratch_B_ = nb;
        free_graphs();
    }
}

// Grid of a persistent pass: `per_sm` CTAs per SM, but no more CTAs than
// there are work items (`items` split into `per_cta` per CTA).
static int pgrid(int sms, int per_sm, uint64_t items, uint64_t per_cta) {
    const uint64_t need = (items + per_cta - 1) / per_cta;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * per_sm, need));
}

void Engine::enqueue_step(bool sets, cudaEvent_t* ev) {
    device_ahead_ = true;
    const int nfl = (int)table_h_.size();
    const int sblocks = pgrid(num_sms_, shape_.stream_blocks_per_sm, V_, 256);
    const uint32_t ntiles = Btot_ / SCAN_TILE;
    if (ev) FLK_CUDA(cudaEventRecord(ev[0], stream_));
    k_hash_count<<<sblocks, 256, 0, stream_>>>(table_d_, nfl, V_, A_, key_, arrival_, counts_, occ_, ctl_);
    if (ev) FLK_CUDA(cudaEventRecord(ev[1], stream_));
    k_scan<<<ntiles, SCAN_THREADS, 0, stream_>>>(counts_, offsets_, ntiles, status_, ctl_);
    if (ev) FLK_CUDA(cudaEventRecord(ev[2], stream_));
    k_scatter<<<sblocks, 256, 0, stream_>>>(table_d_, nfl, V_, key_, arrival_, offsets_, tmp_, ctl_);
    k_segsort<<<pgrid(num_sms_, shape_.segsort_blocks_per_sm, V_, 8), 256, 0, stream_>>>(
        table_d_, nfl, V_, ctl_, occ_, offsets_, tmp_, A_, B_, D_, sorted_, spos_, sfwd_, due_);
    if (ev) FLK_CUDA(cudaEventRecord(ev[3], stream_));
    const int dblocks = pgrid(num_sms_, shape_.decide_blocks_per_sm, V_, shape_.decide_threads / 32);
    if (sets)
        k_decide<true><<<dblocks, shape_.decide_threads, 0, stream_>>>(table_d_, V_, ctl_, due_, offsets_, spos_, sfwd_,
                                                                       B_, C_, D_, radius_table_, sets_);
    else
        k_decide<false><<<dblocks, shape_.decide_threads, 0, stream_>>>(table_d_, V_, ctl_, due_, offsets_, spos_,
                                                                        sfwd_, B_, C_, D_, radius_table_, nullptr);
    if (ev) FLK_CUDA(cudaEventRecord(ev[4], stream_));
    k_integrate<<<sblocks, 256, 0, stream_>>>(table_d_, nfl, V_, A_, B_, C_, ctl_);
    if (ev) FLK_CUDA(cudaEventRecord(ev[5], stream_));
}

void Engine::ensure_graph() {
    const uint32_t chunk = (uint32_t)std::max(1, shape_.graph_chunk);
    if (graph_ && graph_steps_ == chunk) return;
    free_graphs();
    cudaGraph_t g;
    FLK_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    for (uint32_t s = 0; s < chunk; ++s) enqueue_step(false);
    FLK_CUDA(cudaStreamEndCapture(stream_, &g));
    cudaError_t e = cudaGraphInstantiate(&graph_, g, 0);
    cudaGraphDestroy(g);
    FLK_CUDA(e);
    graph_steps_ = chunk;
}

void Engine::run(uint32_t steps) {
    FLK_CUDA(cudaSetDevice(device_));
    if (table_dirty_) {
        sync_times();
        rebuild_table();
    }
    if (table_h_.empty() || steps == 0) return;
    const uint32_t chunk = (uint32_t)std::max(1, shape_.graph_chunk);
    uint32_t done = 0;
    if (steps >= chunk) {
        ensure_graph();
        device_ahead_ = true;
        for (; done + chunk <= steps; done += chunk) FLK_CUDA(cudaGraphLaunch(graph_, stream_));
    }
    for (; done < steps; ++done) enqueue_step(false);
    FLK_CUDA(cudaGetLastError());
    // host mirror of the countdown (clocks are read back on demand)
    bool finished = false;
    for (size_t k = 0; k < table_h_.size(); ++k) {
        const uint32_t left = table_h_[k].remaining > steps ? table_h_[k].remaining - steps : 0;
        table_h_[k].remaining = left;
        if (table_ids_[k] >= 0) slots_[table_ids_[k]].remaining = left;
        finished |= left == 0;
    }
    // flocks that reached zero leave the table at the next run (their clocks
    // are read back from the device table before it is rebuilt)
    if (finished) table_dirty_ = true;
}

void Engine::run_timed(uint32_t steps, uint32_t warmup, PassTimes* out) {
    FLK_CUDA(cudaSetDevice(device_));
    if (table_dirty_) {
        sync_times();
        rebuild_table();
    }
    PassTimes pt{};
    if (table_h_.empty() || steps == 0) {
        if (out) *out = pt;
        return;
    }
    std::vector<cudaEvent_t> ev((size_t)steps * 6);
    for (auto& e : ev) FLK_CUDA(cudaEventCreate(&e));
    for (uint32_t s = 0; s < steps; ++s) enqueue_step(false, &ev[(size_t)s * 6]);
    FLK_CUDA(cudaGetLastError());
    FLK_CUDA(cudaStreamSynchronize(stream_));
    warmup = std::min(warmup, steps);
    for (uint32_t s = warmup; s < steps; ++s) {
        cudaEvent_t* e = &ev[(size_t)s * 6];
        for (int p = 0; p < 5; ++p) {
            float ms = 0;
            FLK_CUDA(cudaEventElapsedTime(&ms, e[p], e[p + 1]));
            pt.ms[p] += ms;
        }
    }
    pt.timed_steps = (int)(steps - warmup);
    if (pt.timed_steps > 0) {
        for (int p = 0; p < 5; ++p) {
            pt.ms[p] /= pt.timed_steps;
            pt.total_ms += pt.ms[p];
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    sync_times();  // clocks and countdowns from the device table
    table_dirty_ = true;
    if (out) *out = pt;
}

void Engine::step_debug(std::vector<GridDebug>* out) {
    FLK_CUDA(cudaSetDevice(device_));
    if (table_dirty_) {
        sync_times();
        rebuild_table();
    }
    if (table_h_.empty()) return;
    if (!sets_) sets_ = dalloc<uint32_t>((size_t)scratch_V_ * 8, &dev_bytes_);
    FLK_CUDA(cudaMemsetAsync(sets_, 0, (size_t)V_ * 8 * 4, stream_));
    const std::vector<FlockDesc> before = table_h_;
    enqueue_step(true);
    FLK_CUDA(cudaGetLastError());
    FLK_CUDA(cudaStreamSynchronize(stream_));
    std::vector<uint32_t> key(V_), offs((size_t)Btot_ + 1), sorted(V_), sets((size_t)V_ * 8);
    FLK_CUDA(cudaMemcpy(key.data(), key_, (size_t)V_ * 4, cudaMemcpyDeviceToHost));
    FLK_CUDA(cudaMemcpy(offs.data(), offsets_, ((size_t)Btot_ + 1) * 4, cudaMemcpyDeviceToHost));
    FLK_CUDA(cudaMemcpy(sorted.data(), sorted_, (size_t)V_ * 4, cudaMemcpyDeviceToHost));
    FLK_CUDA(cudaMemcpy(sets.data(), sets_, (size_t)V_ * 8 * 4, cudaMemcpyDeviceToHost));
    out->clear();
    for (const FlockDesc& d : before) {
        GridDebug g;
        g.keys.resize(d.n);
        for (uint32_t i = 0; i < d.n; ++i) g.keys[i] = key[d.vbase + i] - d.bbase;
        g.offsets.resize((size_t)d.buckets + 1);
        const uint32_t o0 = offs[d.bbase];
        for (uint32_t b = 0; b <= d.buckets; ++b) g.offsets[b] = offs[(size_t)d.bbase + b] - o0;
        g.sorted.assign(sorted.begin() + o0, sorted.begin() + o0 + d.n);
        g.sets.assign(sets.begin() + (size_t)d.vbase * 8, sets.begin() + (size_t)(d.vbase + d.n) * 8);
        out->push_back(std::move(g));
    }
    sync_times();  // clocks and countdowns from the device table
    table_dirty_ = true;
}

void Engine::sync() {
    FLK_CUDA(cudaSetDevice(device_));
    FLK_CUDA(cudaStreamSynchronize(stream_));
}

uint32_t Engine::check_device_error() {
    FLK_CUDA(cudaSetDevice(device_));
    StepCtl c;
    FLK_CUDA(cudaMemcpyAsync(&c, ctl_, sizeof c, cudaMemcpyDeviceToHost, stream_));
    FLK_CUDA(cudaStreamSynchronize(stream_));
    if (c.error) {
        const uint32_t z = 0;
        FLK_CUDA(cudaMemcpyAsync(&ctl_->error, &z, 4, cudaMemcpyHostToDevice, stream_));
        FLK_CUDA(cudaStreamSynchronize(stream_));
    }
    return c.error;
}

void Engine::counters(unsigned long long* due, unsigned long long* cand, unsigned long long* pairs) {
    FLK_CUDA(cudaSetDevice(device_));
    StepCtl c;
    FLK_CUDA(cudaMemcpyAsync(&c, ctl_, sizeof c, cudaMemcpyDeviceToHost, stream_));
    FLK_CUDA(cudaStreamSynchronize(stream_));
    if (due) *due = c.due_total;
    if (cand) *cand = c.cand_total;
    if (pairs) *pairs = c.pair_total;
}

}  // namespace flk
