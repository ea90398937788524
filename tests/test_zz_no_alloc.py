"""flk_grid_noalloc: the grid build for callers that cannot allocate device memory.

Some hosts own all device memory (their own pool, a fixed budget, a real-time
loop that cannot take cudaMalloc's implicit synchronisation) and only hand a
library device buffers. This test plays such a caller: it allocates the input
and output buffers itself, calls the entry point through the C ABI twice in a
row (a larger flock, then a smaller one, so leftovers in the shared scratch
would show), and checks each result against flk_step_debug's grid for the same
positions. Grid outputs are integers, so the tolerance is zero: bit-exact.

This file is collected last so that a run that stops at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class DeviceBuffers:
    """Caller-owned device memory through the CUDA driver API (not the library)."""

    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        self._ck(self.cu.cuInit(0))
        dev = C.c_int()
        self._ck(self.cu.cuDeviceGet(C.byref(dev), 0))
        self.dev = dev
        self.ctx = C.c_void_p()
        self._ck(self.cu.cuDevicePrimaryCtxRetain(C.byref(self.ctx), dev))
        self._ck(self.cu.cuCtxSetCurrent(self.ctx))
        self.ptrs = []

    @staticmethod
    def _ck(rc):
        assert rc == 0, f"CUDA driver error {rc}"

    def alloc(self, nbytes: int) -> int:
        p = C.c_uint64()
        self._ck(self.cu.cuMemAlloc_v2(C.byref(p), C.c_size_t(max(nbytes, 16))))
        self.ptrs.append(p.value)
        return p.value

    def upload(self, a: np.ndarray) -> int:
        p = self.alloc(a.nbytes)
        self._ck(self.cu.cuMemcpyHtoD_v2(C.c_uint64(p), a.ctypes.data_as(C.c_void_p), C.c_size_t(a.nbytes)))
        return p

    def download(self, p: int, count: int, dtype=np.uint32) -> np.ndarray:
        out = np.zeros(count, dtype=dtype)
        self._ck(self.cu.cuMemcpyDtoH_v2(out.ctypes.data_as(C.c_void_p), C.c_uint64(p), C.c_size_t(out.nbytes)))
        return out

    def free(self):
        for p in self.ptrs:
            self.cu.cuMemFree_v2(C.c_uint64(p))
        self.ptrs = []
        if self.ctx:
            # balances the retain above (the runtime holds its own reference)
            self.cu.cuDevicePrimaryCtxRelease_v2(self.dev)
            self.ctx = None


def grid_noalloc(native, bufs, words):
    L = native.lib()
    fn = L.flk_grid_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint64, C.c_void_p]
    n = len(words)
    B = native.buckets_for(n)
    pos4 = np.zeros((n, 4), dtype=np.float32)
    pos4[:, :3] = words[:, :3]
    d_pos = bufs.upload(pos4)
    d_keys, d_offs, d_sorted = bufs.alloc(n * 4), bufs.alloc((B + 1) * 4), bufs.alloc(n * 4)
    rc = fn(d_pos, n, d_keys, d_offs, d_sorted, None)
    assert rc == 0, L.flk_last_error()
    return bufs.download(d_keys, n), bufs.download(d_offs, B + 1), bufs.download(d_sorted, n)


def test_grid_noalloc_equals_flk_step_debug_on_two_calls_in_a_row(native):
    bufs = DeviceBuffers()
    try:
        for n, seed in [(131_072, 1), (3_000, 9)]:
            words = native.generate(n, seed)
            f = native.Flock(words)
            want = f.step_debug()  # the existing entry point's grid for these positions
            f.close()
            keys, offs, srt = grid_noalloc(native, bufs, words)
            assert np.array_equal(keys, want["keys"]), n
            assert np.array_equal(offs, want["offsets"]), n
            assert np.array_equal(srt, want["sorted"]), n
    finally:
        bufs.free()


def test_grid_noalloc_of_an_empty_flock_writes_every_offset(native):
    # n = 0 still has buckets_for(0) = 65,536 buckets: all 65,537 offsets are written as 0
    bufs = DeviceBuffers()
    try:
        B = native.buckets_for(0)
        assert B == 1 << 16
        L = native.lib()
        fn = L.flk_grid_noalloc
        fn.restype = C.c_int
        fn.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint64, C.c_void_p]
        d_offs = bufs.upload(np.full(B + 1, 0xDEADBEEF, dtype=np.uint32))
        d_pos = bufs.alloc(16)
        rc = fn(d_pos, 0, 0, d_offs, 0, None)
        assert rc == 0, L.flk_last_error()
        assert np.array_equal(bufs.download(d_offs, B + 1), np.zeros(B + 1, dtype=np.uint32))
    finally:
        bufs.free()


def test_grid_noalloc_rejects_more_birds_than_its_scratch_holds(native):
    L = native.lib()
    fn = L.flk_grid_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint64, C.c_void_p]
    rc = fn(16, 131_073, 16, 16, 16, None)  # rejected before any device work
    assert rc == -5
    assert b"exceeds the maximum of 131072" in L.flk_last_error()
