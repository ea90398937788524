// flk_grid_noalloc: the grid build of one flock step (cell keys, bucket
// offsets, stable sorted order) for callers that cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is off limits -- a host
// application that owns every byte of device memory through its own pool and
// forbids libraries from allocating behind its back, a real-time loop where
// cudaMalloc's implicit device synchronisation would stall the frame, or a
// plugin loaded into a process whose memory budget is fixed up front. Such a
// caller hands in device buffers for the inputs and outputs; everything else
// the passes need (histogram, arrival ranks, the unsorted slots, the
// occupied-bucket list, the scan's tile flags and counters) lives in one
// file-scope device array, g_flk_noalloc_scratch, sized for at most
// FLK_NOALLOC_MAX_BIRDS birds. Every GPU that loads this library holds that
// array (about 2.5 MiB) until the process exits.
//
// The array's name in host code is only a host-side handle, not a device
// address, so every call looks the address up with cudaGetSymbolAddress on the
// current device and passes the pointer to the kernels. Nothing is cached
// across calls, so a device reset between calls (which reloads the module and
// moves the array) cannot leave a stale address behind. The call is blocking:
// it synchronises its stream before it returns.
//
// All calls share the one array and it keeps the previous call's contents:
// each call clears the parts that must start at zero. Calls that overlap on the
// GPU (different streams or threads, same device) race on the array and give
// wrong results; serialise them.
//
// The passes restate the engine's hash/count, decoupled look-back scan,
// scatter and per-bucket stable sort for a single flock, so the outputs equal
// flk_step_debug's keys/offsets/sorted bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>

#include "../../include/flock_gb300.h"
#include "flock_params.h"

namespace flk {
void set_last_error(const std::string& msg);  // flock_abi.cpp
}

namespace {

constexpr uint32_t MAX_BIRDS = FLK_NOALLOC_MAX_BIRDS;
constexpr uint32_t MAX_BUCKETS = 2u * FLK_NOALLOC_MAX_BIRDS;  // buckets_for(MAX_BIRDS)
constexpr uint32_t TILE = 4096;                               // buckets per scan tile
constexpr uint32_t MAX_TILES = MAX_BUCKETS / TILE;
constexpr uint32_t SPIN_LIMIT = 1u << 22;
constexpr uint32_t FULL = 0xFFFFFFFFu;

// Byte layout of the scratch array (each region 256-byte aligned).
constexpr size_t OFF_COUNTS = 0;                                  // MAX_BUCKETS u32
constexpr size_t OFF_ARRIVAL = OFF_COUNTS + MAX_BUCKETS * 4ull;   // MAX_BIRDS u32
constexpr size_t OFF_TMP = OFF_ARRIVAL + MAX_BIRDS * 4ull;        // MAX_BIRDS u32
constexpr size_t OFF_OCC = OFF_TMP + MAX_BIRDS * 4ull;            // MAX_BIRDS u32
constexpr size_t OFF_STATUS = OFF_OCC + MAX_BIRDS * 4ull;         // MAX_TILES u64
constexpr size_t OFF_CTL = OFF_STATUS + MAX_TILES * 8ull;         // 16 u32
constexpr size_t SCRATCH_BYTES = OFF_CTL + 256;
enum { CTL_OCC = 0, CTL_TICKET = 1, CTL_ERROR = 2 };

static_assert(OFF_STATUS % 256 == 0 && OFF_CTL % 256 == 0, "scratch regions stay 256-byte aligned");

}  // namespace

static __device__ __align__(256) unsigned char g_flk_noalloc_scratch[SCRATCH_BYTES];

namespace {

struct Scratch {
    uint32_t* counts;
    uint32_t* arrival;
    uint32_t* tmp;
    uint32_t* occ;
    unsigned long long* status;
    uint32_t* ctl;
};

Scratch carve(unsigned char* base) {
    return Scratch{reinterpret_cast<uint32_t*>(base + OFF_COUNTS), reinterpret_cast<uint32_t*>(base + OFF_ARRIVAL),
                   reinterpret_cast<uint32_t*>(base + OFF_TMP), reinterpret_cast<uint32_t*>(base + OFF_OCC),
                   reinterpret_cast<unsigned long long*>(base + OFF_STATUS),
                   reinterpret_cast<uint32_t*>(base + OFF_CTL)};
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}
__device__ __forceinline__ int cell1(float x) { return (int)floorf(__fmul_rn(x, flk::INV_CELL)); }

__global__ void k_na_hash_count(const float4* __restrict__ pos, uint32_t n, uint32_t mask, uint32_t* __restrict__ keys,
                                Scratch s) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t v0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); v0 < n; v0 += gridDim.x * blockDim.x) {
        const uint32_t v = v0 + lane;
        const bool act = v < n;
        uint32_t b = 0;
        if (act) {
            const float4 p = pos[v];
            b = (((uint32_t)cell1(p.x) * 73856093u) ^ ((uint32_t)cell1(p.y) * 19349663u) ^
                 ((uint32_t)cell1(p.z) * 83492791u)) & mask;
            keys[v] = b;
        }
        const uint32_t m = __ballot_sync(FULL, act);
        if (act) {
            const uint32_t peers = __match_any_sync(m, b);
            const int leader = __ffs(peers) - 1;
            uint32_t old = 0;
            if ((int)lane == leader) old = atomicAdd(&s.counts[b], (uint32_t)__popc(peers));
            old = __shfl_sync(m, old, leader);
            const uint32_t rank = old + __popc(peers & lanemask_lt());
            s.arrival[v] = rank;
            const bool first = rank == 0;
            const uint32_t fm = __ballot_sync(m, first);
            if (fm) {
                const int wl = __ffs(m) - 1;
                uint32_t base = 0;
                if ((int)lane == wl) base = atomicAdd(&s.ctl[CTL_OCC], (uint32_t)__popc(fm));
                base = __shfl_sync(m, base, wl);
                if (first) s.occ[base + __popc(fm & lanemask_lt())] = b;
            }
        }
    }
}

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Exclusive scan of counts[0..ntiles*TILE) into offsets (+ the total), one
// tile of 256 threads x 16 buckets per CTA, decoupled look-back over flags
// (1 = aggregate, 2 = inclusive prefix) that start zeroed each call.
__global__ void __launch_bounds__(256) k_na_scan(uint32_t* __restrict__ offsets, uint32_t ntiles, Scratch s) {
    __shared__ uint32_t s_tile, s_prefix, s_warp[8];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_tile = atomicAdd(&s.ctl[CTL_TICKET], 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) return;
    const size_t base = (size_t)tile * TILE + threadIdx.x * 16;
    uint4 c[4];
    const uint4* src = reinterpret_cast<const uint4*>(s.counts + base);
#pragma unroll
    for (int k = 0; k < 4; ++k) c[k] = src[k];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) sum += c[k].x + c[k].y + c[k].z + c[k].w;
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
    for (int w = 0; w < 8; ++w) {
        if (w < (int)warp) wpre += s_warp[w];
        agg += s_warp[w];
    }
    if (warp == 0) {
        uint32_t excl = 0;
        if (tile == 0) {
            if (lane == 0) st_relaxed(&s.status[0], (2ull << 32) | agg);
        } else {
            if (lane == 0) st_relaxed(&s.status[tile], (1ull << 32) | agg);
            int pred = (int)tile - 1;
            uint32_t polls = 0;
            while (true) {
                const int idx = pred - (int)lane;
                uint32_t flag = 2, val = 0;
                while (true) {
                    if (idx >= 0) {
                        const unsigned long long w = ld_relaxed(&s.status[idx]);
                        flag = (uint32_t)(w >> 32);
                        val = (uint32_t)w;
                    }
                    if (__all_sync(FULL, flag != 0)) break;
                    if (++polls > SPIN_LIMIT) {  // give up, record, and let every waiter finish
                        if (lane == 0) atomicCAS(&s.ctl[CTL_ERROR], 0u, 1u);
                        flag = 2;
                        val = 0;
                        break;
                    }
                    __nanosleep(64);
                }
                const uint32_t pm = __ballot_sync(FULL, flag == 2);
                const int firstp = pm ? __ffs(pm) - 1 : 32;
                uint32_t x = ((int)lane <= firstp) ? val : 0u;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
                excl += x;
                if (pm) break;
                pred -= 32;
            }
            if (lane == 0) st_relaxed(&s.status[tile], (2ull << 32) | (excl + agg));
        }
        if (lane == 0) s_prefix = excl;
    }
    __syncthreads();
    uint32_t run = s_prefix + wpre + inc - sum;
    uint4* dst = reinterpret_cast<uint4*>(offsets + base);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        uint4 o;
        o.x = run; run += c[k].x;
        o.y = run; run += c[k].y;
        o.z = run; run += c[k].z;
        o.w = run; run += c[k].w;
        dst[k] = o;
    }
    if (tile == ntiles - 1 && threadIdx.x == 255) offsets[(size_t)ntiles * TILE] = run;
}

__global__ void k_na_scatter(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ offsets, uint32_t n,
                             Scratch s) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t pos = offsets[keys[v]] + s.arrival[v];
        if (pos < n) s.tmp[pos] = v;
        else atomicCAS(&s.ctl[CTL_ERROR], 0u, 2u);
    }
}

// One warp per occupied bucket: its slots sorted by bird index.
__global__ void k_na_segsort(const uint32_t* __restrict__ offsets, uint32_t n, uint32_t* __restrict__ sorted,
                             Scratch s) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nocc = *(volatile uint32_t*)&s.ctl[CTL_OCC];
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nocc; w += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t b = s.occ[w];
        const uint32_t s0 = offsets[b], e0 = offsets[b + 1];
        if (e0 < s0 || e0 > n) {
            if (lane == 0) atomicCAS(&s.ctl[CTL_ERROR], 0u, 2u);
            continue;
        }
        const uint32_t L = e0 - s0;
        if (L <= 32) {
            uint32_t x = lane < L ? s.tmp[s0 + lane] : 0xFFFFFFFFu;
#pragma unroll
            for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
                for (int j = k >> 1; j > 0; j >>= 1) {
                    const uint32_t y = __shfl_xor_sync(FULL, x, j);
                    const bool up = (lane & k) == 0, lower = (lane & j) == 0;
                    x = (lower == up) ? min(x, y) : max(x, y);
                }
            }
            if (lane < L) sorted[s0 + lane] = x;
        } else {
            for (uint32_t c0 = 0; c0 < L; c0 += 32) {
                const bool has = c0 + lane < L;
                const uint32_t x = has ? s.tmp[s0 + c0 + lane] : 0xFFFFFFFFu;
                uint32_t rank = 0;
                for (uint32_t j0 = 0; j0 < L; j0 += 32) {
                    const uint32_t y = (j0 + lane < L) ? s.tmp[s0 + j0 + lane] : 0xFFFFFFFFu;
                    for (int q = 0; q < 32; ++q) rank += __shfl_sync(FULL, y, q) < x;
                }
                if (has) sorted[s0 + rank] = x;
            }
        }
    }
}

int na_fail(int code, const std::string& m) {
    flk::set_last_error(m);  // reported by flk_last_error()
    return code;
}

}  // namespace

extern "C" int flk_grid_noalloc(const float* pos4, uint32_t n, uint32_t* keys, uint32_t* offsets, uint32_t* sorted,
                                void* stream) {
    if (n > MAX_BIRDS)
        return na_fail(FLK_ERR_CAPACITY, "flk_grid_noalloc: " + std::to_string(n) + " birds exceeds the maximum of " +
                                             std::to_string(MAX_BIRDS) + " this entry point's fixed scratch holds");
    if (!offsets || (n && (!pos4 || !keys || !sorted)))
        return na_fail(FLK_ERR_ARG, "flk_grid_noalloc: null device pointer");
    // float4 loads of pos4 and 16-byte stores into offsets need 16-byte alignment
    if ((reinterpret_cast<uintptr_t>(pos4) | reinterpret_cast<uintptr_t>(offsets)) & 15u)
        return na_fail(FLK_ERR_ARG, "flk_grid_noalloc: pos4 and offsets must be 16-byte aligned");
    // the scratch array's device address on the current device, looked up on
    // every call (cheap next to the stream synchronisation below)
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_flk_noalloc_scratch);
    if (e != cudaSuccess) return na_fail(FLK_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    unsigned char* base = static_cast<unsigned char*>(p);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint64_t want = 1;
    while (want < (uint64_t)n * 2) want <<= 1;
    const uint32_t B = (uint32_t)(want < (1u << 16) ? (1u << 16) : want);  // n <= MAX_BIRDS keeps B <= 2^22
    const uint32_t ntiles = B / TILE;
    const Scratch s = carve(base);
    // what must start at zero: the histogram, the scan flags and the counters
    e = cudaMemsetAsync(s.counts, 0, (size_t)B * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.status, 0, (size_t)ntiles * 8, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.ctl, 0, 64, st);
    if (e != cudaSuccess) return na_fail(FLK_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    const int blocks = (int)std::min<uint32_t>(std::max<uint32_t>((n + 255) / 256, 1u), 1024u);
    k_na_hash_count<<<blocks, 256, 0, st>>>(reinterpret_cast<const float4*>(pos4), n, B - 1, keys, s);
    k_na_scan<<<ntiles, 256, 0, st>>>(offsets, ntiles, s);
    k_na_scatter<<<blocks, 256, 0, st>>>(keys, offsets, n, s);
    const int sblocks = (int)std::min<uint32_t>(std::max<uint32_t>((n + 7) / 8, 1u), 2048u);
    k_na_segsort<<<sblocks, 256, 0, st>>>(offsets, n, sorted, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return na_fail(FLK_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    uint32_t err = 0;
    e = cudaMemcpyAsync(&err, s.ctl + CTL_ERROR, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return na_fail(FLK_ERR_CUDA, std::string("flk_grid_noalloc: ") + cudaGetErrorString(e));
    if (err) return na_fail(FLK_ERR_DEVICE, "flk_grid_noalloc: device error word " + std::to_string(err));
    return FLK_OK;
}
