"""The reference's own CUDA kernels, driven through the CUDA driver API.

Test and reference-timing infrastructure only: used by tests/golden/make_reference_fixtures.py
(golden fixtures) and by bench.py's reference-kernel baseline. The product
package never imports it.

The reference's cuda/flock.cu is compiled unchanged for sm_103a into
oracle/_ref/flock_ref_sm103a.cubin (oracle/Makefile, target `ref`, built only
where the reference project is mounted). This module loads that cubin and drives
its kernels exactly as the reference's host loop does (cuda/flock.cu:403-470:
buckets_for, memset, grid_histogram, the three scan kernels, grid_scatter,
decide, integrate, one stream, time += DT in f32 on the host), with the
reference's timing protocol (cuda/flock.cu:447-492: CUDA events between passes,
mean GPU ms per pass over the timed steps).

Safety: before any launch it checks each kernel's parameter layout with
cuFuncGetParamInfo against the struct built here, and aborts on a mismatch.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "flock_ref_sm103a.cubin")

DT = np.float32(0.005)
SCAN_BLOCK = 2048  # cuda/flock.cu:113-115


class FlockArg(C.Structure):
    """cuda/flock.cu:93-111, passed by value to every kernel."""
    _fields_ = [("n", C.c_int), ("buckets", C.c_uint32)] + [
        (k, C.c_uint64) for k in ("pos", "vel", "steer", "roll", "spin", "radius", "next_decision", "centrality",
                                  "neighbours", "bucket", "counts", "offsets", "block_sums", "sorted")]


class Driver:
    def __init__(self, device: int = 0):
        if not os.path.exists(CUBIN):
            raise FileNotFoundError(CUBIN + " (built by `make -C oracle ref` where the reference is mounted)")
        self.cu = C.CDLL("libcuda.so.1")
        self.ck(self.cu.cuInit(0))
        dev = C.c_int()
        self.ck(self.cu.cuDeviceGet(C.byref(dev), device))
        self.dev = dev
        self.ctx = C.c_void_p()
        self.ck(self.cu.cuDevicePrimaryCtxRetain(C.byref(self.ctx), dev))
        self.ck(self.cu.cuCtxSetCurrent(self.ctx))
        self.mod = C.c_void_p()
        self.ck(self.cu.cuModuleLoad(C.byref(self.mod), CUBIN.encode()))
        self.allocs = []

    def ck(self, rc):
        if rc != 0:
            name = C.c_char_p()
            self.cu.cuGetErrorName(rc, C.byref(name))
            raise RuntimeError(f"CUDA driver error {rc} {name.value}")

    def fn(self, mangled: str, sizes: list[int]):
        f = C.c_void_p()
        self.ck(self.cu.cuModuleGetFunction(C.byref(f), self.mod, mangled.encode()))
        off, size = C.c_size_t(), C.c_size_t()
        for i, want in enumerate(sizes):
            self.ck(self.cu.cuFuncGetParamInfo(f, C.c_size_t(i), C.byref(off), C.byref(size)))
            if size.value != want:
                raise RuntimeError(f"{mangled}: parameter {i} is {size.value} bytes, expected {want}")
        if self.cu.cuFuncGetParamInfo(f, C.c_size_t(len(sizes)), C.byref(off), C.byref(size)) == 0:
            raise RuntimeError(f"{mangled}: more parameters than expected")
        return f

    def alloc(self, nbytes: int) -> int:
        p = C.c_uint64()
        self.ck(self.cu.cuMemAlloc_v2(C.byref(p), C.c_size_t(max(nbytes, 4))))
        self.allocs.append(p.value)
        return p.value

    def h2d(self, dst: int, a: np.ndarray):
        a = np.ascontiguousarray(a)
        self.ck(self.cu.cuMemcpyHtoD_v2(C.c_uint64(dst), a.ctypes.data_as(C.c_void_p), C.c_size_t(a.nbytes)))

    def d2h(self, a: np.ndarray, src: int):
        self.ck(self.cu.cuMemcpyDtoH_v2(a.ctypes.data_as(C.c_void_p), C.c_uint64(src), C.c_size_t(a.nbytes)))

    def zero(self, dst: int, words: int):
        self.ck(self.cu.cuMemsetD32_v2(C.c_uint64(dst), C.c_uint(0), C.c_size_t(words)))

    def launch(self, f, grid: int, block: int, args: list):
        ptrs = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        self.ck(self.cu.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, None, ptrs, None))

    def sync(self):
        self.ck(self.cu.cuCtxSynchronize())

    def free(self):
        for p in self.allocs:
            self.cu.cuMemFree_v2(C.c_uint64(p))
        self.allocs = []

    def close(self):
        """Frees the buffers, unloads the module, releases the primary context."""
        self.free()
        if self.mod:
            self.cu.cuModuleUnload(self.mod)
            self.mod = None
        if self.ctx:
            self.cu.cuDevicePrimaryCtxRelease_v2(self.dev)
            self.ctx = None


def buckets_for(n: int) -> int:  # cuda/flock.cu:368-372
    want = 1
    while want < n * 2:
        want <<= 1
    return min(max(want, 1 << 16), 1 << 22)


def run_reference(drv: Driver, words: np.ndarray, time: float, steps: int):
    """The reference's main(): upload (flock.cu:414-437), step loop (453-470),
    download (494-519). Returns (time, words, keys of step 1, offsets of step 1)."""
    n = len(words)
    B = buckets_for(n)
    szF = C.sizeof(FlockArg)
    k_hist = drv.fn("_Z14grid_histogram5Flock", [szF])
    k_sblk = drv.fn("_Z16grid_scan_blocks5Flock", [szF])
    k_stot = drv.fn("_Z16grid_scan_totals5Flockj", [szF, 4])
    k_sadd = drv.fn("_Z13grid_scan_add5Flock", [szF])
    k_scat = drv.fn("_Z12grid_scatter5Flock", [szF])
    k_dec = drv.fn("_Z6decide5Flockf", [szF, 4])
    k_int = drv.fn("_Z9integrate5Flock", [szF])
    f = FlockArg()
    f.n, f.buckets = n, B
    for k in ("pos", "vel", "steer"):
        setattr(f, k, drv.alloc(n * 16))
    for k in ("roll", "spin", "radius", "next_decision", "centrality", "neighbours", "bucket", "sorted"):
        setattr(f, k, drv.alloc(n * 4))
    f.counts = drv.alloc(B * 4)
    f.offsets = drv.alloc((B + 1) * 4)
    f.block_sums = drv.alloc((B // SCAN_BLOCK) * 4)
    w = words.astype(np.float32)
    f4 = lambda cols: np.concatenate([w[:, cols], np.zeros((n, 1), np.float32)], axis=1)
    drv.h2d(f.pos, f4([0, 1, 2]))
    drv.h2d(f.vel, f4([3, 4, 5]))
    drv.h2d(f.steer, f4([9, 10, 11]))
    for k, col in (("roll", 6), ("spin", 7), ("radius", 8), ("next_decision", 12), ("neighbours", 13),
                   ("centrality", 14)):
        drv.h2d(getattr(f, k), np.ascontiguousarray(w[:, col]))
    TB = 256
    blocks = (n + TB - 1) // TB
    scan_blocks = C.c_uint32(B // SCAN_BLOCK)
    t = np.float32(time)
    keys1 = offs1 = None
    for s in range(steps):
        t = np.float32(t + DT)
        drv.zero(f.counts, B)
        drv.launch(k_hist, blocks, TB, [f])
        drv.launch(k_sblk, B // SCAN_BLOCK, 256, [f])
        drv.launch(k_stot, 1, 256, [f, scan_blocks])
        drv.launch(k_sadd, (B + TB - 1) // TB, TB, [f])
        drv.launch(k_scat, blocks, TB, [f])
        drv.launch(k_dec, blocks, TB, [f, C.c_float(float(t))])
        drv.launch(k_int, blocks, TB, [f])
        if s == 0:
            drv.sync()
            keys1 = np.zeros(n, np.uint32)
            offs1 = np.zeros(B + 1, np.uint32)
            drv.d2h(keys1, f.bucket)
            drv.d2h(offs1, f.offsets)
    drv.sync()
    out = np.zeros((n, 15), np.float32)
    tmp4 = np.zeros((n, 4), np.float32)
    for k, cols in (("pos", [0, 1, 2]), ("vel", [3, 4, 5]), ("steer", [9, 10, 11])):
        drv.d2h(tmp4, getattr(f, k))
        out[:, cols] = tmp4[:, :3]
    tmp = np.zeros(n, np.float32)
    for k, col in (("roll", 6), ("spin", 7), ("radius", 8), ("next_decision", 12), ("neighbours", 13),
                   ("centrality", 14)):
        drv.d2h(tmp, getattr(f, k))
        out[:, col] = tmp
    drv.free()
    return float(t), out, keys1, offs1


def time_reference(drv: Driver, n: int, seed: int, steps: int, warmup: int, words=None) -> dict:
    """The reference's own timing protocol (cuda/flock.cu:447-492): per-pass CUDA
    events around the same launches, mean GPU ms per pass over the timed steps.
    `words` (n x 15 float32, the reference generator's scatter of n birds with
    `seed`) defaults to the oracle's generator."""
    if words is None:
        from oracle import pyoracle as o

        words = o.scatter(n, seed)
    words = np.ascontiguousarray(words, dtype=np.float32)
    B = buckets_for(n)
    szF = C.sizeof(FlockArg)
    ks = [drv.fn(m, s) for m, s in (("_Z14grid_histogram5Flock", [szF]), ("_Z16grid_scan_blocks5Flock", [szF]),
                                     ("_Z16grid_scan_totals5Flockj", [szF, 4]), ("_Z13grid_scan_add5Flock", [szF]),
                                     ("_Z12grid_scatter5Flock", [szF]), ("_Z6decide5Flockf", [szF, 4]),
                                     ("_Z9integrate5Flock", [szF]))]
    f = FlockArg()
    f.n, f.buckets = n, B
    for k in ("pos", "vel", "steer"):
        setattr(f, k, drv.alloc(n * 16))
    for k in ("roll", "spin", "radius", "next_decision", "centrality", "neighbours", "bucket", "sorted"):
        setattr(f, k, drv.alloc(n * 4))
    f.counts = drv.alloc(B * 4)
    f.offsets = drv.alloc((B + 1) * 4)
    f.block_sums = drv.alloc((B // SCAN_BLOCK) * 4)
    w = words
    f4 = lambda cols: np.concatenate([w[:, cols], np.zeros((n, 1), np.float32)], axis=1)
    drv.h2d(f.pos, f4([0, 1, 2]))
    drv.h2d(f.vel, f4([3, 4, 5]))
    drv.h2d(f.steer, f4([9, 10, 11]))
    for k, col in (("roll", 6), ("spin", 7), ("radius", 8), ("next_decision", 12), ("neighbours", 13),
                   ("centrality", 14)):
        drv.h2d(getattr(f, k), np.ascontiguousarray(w[:, col]))
    ev = [[C.c_void_p() for _ in range(6)] for _ in range(steps)]
    for row in ev:
        for e in row:
            drv.ck(drv.cu.cuEventCreate(C.byref(e), 0))
    TB = 256
    blocks = (n + TB - 1) // TB
    nblk = C.c_uint32(B // SCAN_BLOCK)
    t = np.float32(0.0)
    for s in range(steps):
        e = ev[s]
        t = np.float32(t + DT)
        drv.ck(drv.cu.cuEventRecord(e[0], None))
        drv.zero(f.counts, B)
        drv.launch(ks[0], blocks, TB, [f])
        drv.ck(drv.cu.cuEventRecord(e[1], None))
        drv.launch(ks[1], B // SCAN_BLOCK, 256, [f])
        drv.launch(ks[2], 1, 256, [f, nblk])
        drv.launch(ks[3], (B + TB - 1) // TB, TB, [f])
        drv.ck(drv.cu.cuEventRecord(e[2], None))
        drv.launch(ks[4], blocks, TB, [f])
        drv.ck(drv.cu.cuEventRecord(e[3], None))
        drv.launch(ks[5], blocks, TB, [f, C.c_float(float(t))])
        drv.ck(drv.cu.cuEventRecord(e[4], None))
        drv.launch(ks[6], blocks, TB, [f])
        drv.ck(drv.cu.cuEventRecord(e[5], None))
    drv.sync()
    names = ["grid_histogram", "grid_scan", "grid_scatter", "decide", "integrate"]
    tot = [0.0] * 5
    ms = C.c_float()
    for s in range(warmup, steps):
        for p in range(5):
            drv.ck(drv.cu.cuEventElapsedTime_v2(C.byref(ms), ev[s][p], ev[s][p + 1]))
            tot[p] += ms.value
    timed = steps - warmup
    out = {nm: tot[p] / timed for p, nm in enumerate(names)}
    out["step_total"] = sum(tot) / timed
    out["bird_steps_per_s"] = n / (out["step_total"] / 1e3)
    for row in ev:
        for e in row:
            drv.cu.cuEventDestroy_v2(e)
    drv.free()
    return out
