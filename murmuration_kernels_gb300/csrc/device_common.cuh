// Device helpers shared by the step's passes: f32 vector arithmetic with
// explicit round-to-nearest operations (no FMA contraction), the reference's
// forward/side/body_up (crates/flock-ref/src/model.rs:15-38), the cell hash
// (cuda/flock.cu:77-83), warp utilities and relaxed loads/stores.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "flock_engine.h"
#include "flock_params.h"

namespace flk {

constexpr uint32_t FULL = 0xFFFFFFFFu;
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr uint32_t SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;  // 4096 buckets per tile
constexpr uint32_t SCAN_SPIN_LIMIT = 1u << 22;             // look-back polls before giving up
constexpr uint32_t FLAG_A = 1u, FLAG_P = 2u;

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
// Cell of coordinate x in a grid of edge 1 / inv_cell: floor(x * inv_cell),
// monotonic in x for any edge; production steps use the same expression in
// every pass (the edge is a runtime choice, the autotuner's `cell` axis).
__device__ __forceinline__ int pcell(float x, float inv_cell) { return (int)floorf(__fmul_rn(x, inv_cell)); }
// The quarter-cell z-slab of z within its cell cz (inv4 = 4 / edge), clamped
// to 0..3 against the rounding of z * inv4 next to a cell boundary; decide's
// slab trim stays conservative, since the slab index and floor(z * inv4)
// move together.
__device__ __forceinline__ uint32_t pslab(float z, int cz, float inv4) {
    return (uint32_t)min(3, max(0, pcell(z, inv4) - 4 * cz));
}
__device__ __forceinline__ uint32_t cell_hash(int cx, int cy, int cz) {
    return ((uint32_t)cx * 73856093u) ^ ((uint32_t)cy * 19349663u) ^ ((uint32_t)cz * 83492791u);
}

// Bucket of a cell in a production step (one that reports no grid). The
// reference hash above sends about a third of a compact flock's cells to a
// bucket shared with another cell (its XOR of products collides on the cell
// lattice), which costs decide a second cell of candidates each time. Here the
// cell's coordinates are taken modulo a 2^bx x 2^by x 2^bz lattice (bx + by +
// bz = log2 buckets, x fastest): cells of a flock narrower than the lattice in
// every axis (512 x 512 x 256 m from the 2^20 buckets of 1M birds) never share
// a bucket, and
// neighbouring cells along x get neighbouring buckets. Wider flocks wrap, and
// a cell then shares its bucket with its lattice translate; results do not
// depend on which cells share buckets.
__device__ __forceinline__ uint32_t lattice_bucket(int cx, int cy, int cz, uint32_t buckets) {
    const uint32_t k = 31u - (uint32_t)__clz(buckets);  // buckets = 2^k, k >= 12: 16+ cells per axis
    const uint32_t bx = (k + 2u) / 3u, by = (k + 1u - bx) >> 1, bz = k - bx - by;
    const uint32_t x = (uint32_t)cx & ((1u << bx) - 1u);
    const uint32_t y = (uint32_t)cy & ((1u << by) - 1u);
    const uint32_t z = (uint32_t)cz & ((1u << bz) - 1u);
    return x | (y << bx) | (z << (bx + by));
}

// The cells a deciding bird at p with radius r visits: the box of cells that
// a search reach of 2r, inflated so that every bird the exact test d2 <= (2r)^2
// accepts lies in a visited cell (covering the rounding of p -/+ reach as
// well), touches. `wide` flags an absurd reach (huge or non-finite radius).
struct SearchBox {
    float reach, reach2;
    int lx, ly, lz;
    long long nx, ny, nz, ncell;
    bool wide;
};
// Cells of edge 1 / inv_cell (the reference's 4 m cells by default).
__device__ __forceinline__ SearchBox search_box(f3 p, float r, float inv_cell = INV_CELL) {
    SearchBox b;
    const float rr = __fmul_rn(2.0f, r);
    const float pm = fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z)));
    b.reach = rr * 1.00001f + 1e-3f + pm * 1e-6f;
    b.reach2 = b.reach * b.reach;
    b.lx = pcell(p.x - b.reach, inv_cell);
    b.ly = pcell(p.y - b.reach, inv_cell);
    b.lz = pcell(p.z - b.reach, inv_cell);
    b.nx = (long long)pcell(p.x + b.reach, inv_cell) - b.lx + 1;
    b.ny = (long long)pcell(p.y + b.reach, inv_cell) - b.ly + 1;
    b.nz = (long long)pcell(p.z + b.reach, inv_cell) - b.lz + 1;
    b.wide = b.nx > (1 << 20) || b.ny > (1 << 20) || b.nz > (1 << 20);
    b.ncell = b.wide ? (1ll << 62) : b.nx * b.ny * b.nz;
    return b;
}

// floor(x / d) = (x * m) >> 16 with m = floor(65536 / d) + 1 holds for x < 32
// and d <= 32 (m exceeds 65536 / d by at most 1, so the error x / 65536 < 1 / d
// never reaches the next integer); floor(65536 / d) from an approximate f32
// quotient is exact here, since 65536 / d is a power of two or at least 1/32
// away from an integer. m < 2^17.
__device__ __forceinline__ uint32_t div_magic(uint32_t d) {
    return __float2uint_rz(__fdividef(65536.0f, (float)d)) + 1u;
}

// The per-axis bit counts of lattice_bucket for `buckets` (a power of two),
// packed as bx | by << 5 | bz << 10.
__device__ __forceinline__ uint32_t lattice_bits(uint32_t buckets) {
    const uint32_t k = 31u - (uint32_t)__clz(buckets);
    const uint32_t bx = (k + 2u) / 3u, by = (k + 1u - bx) >> 1, bz = k - bx - by;
    return bx | (by << 5) | (bz << 10);
}
// lattice_bucket with the bit counts given (bits from lattice_bits)
__device__ __forceinline__ uint32_t lattice_bucket_bits(int cx, int cy, int cz, uint32_t bits) {
    const uint32_t bx = bits & 31u, by = (bits >> 5) & 31u, bz = (bits >> 10) & 31u;
    const uint32_t x = (uint32_t)cx & ((1u << bx) - 1u);
    const uint32_t y = (uint32_t)cy & ((1u << by) - 1u);
    const uint32_t z = (uint32_t)cz & ((1u << bz) - 1u);
    return x | (y << bx) | (z << (bx + by));
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

// Slot - view index of a flock's birds in buffer p (wraps modulo 2^32).
__device__ __forceinline__ uint32_t view_shift(uint32_t sbase, uint32_t vbase, uint32_t p, uint32_t cap) {
    return p * cap + sbase - vbase;
}

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}


}  // namespace flk
