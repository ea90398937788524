"""GB300-native starling-flock step: Python host mirror over the C ABI.

The reference (ImanolGo/murmuration-kernels) drives its GPU step as a program
(`flock_cuda --in F --steps K --warmup W --out F`, cuda/flock.cu:374-523) over
the FLK1 state file (crates/flock-ref/src/state.rs:104-171). This module
exposes the same operations in-process through `include/flock_gb300.h`:

    Flock      one resident flock: step / step_timed / read / write / step_debug
    Batch      many independent flocks advanced in one launch per pass
    Pool       continuous batching of simulate(flock, steps) requests
    generate   the benchmark scatter (state.rs:79-101)
    read_flk / write_flk   the .flk file

The native library must be built (``python -m murmuration_kernels_gb300.build``);
there is no CPU fallback: every call runs the sm_103a kernels or raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libflock_gb300.so")
CLI_PATH = os.path.join(HERE, "_build", "flock_gb300")
HEADER = os.path.join(os.path.dirname(HERE), "include", "flock_gb300.h")
WORDS = 15

FLK_OK = 0
ERRORS = {-1: "ARG", -2: "IO", -3: "CUDA", -4: "ID", -5: "CAPACITY", -6: "DEVICE", -7: "FORMAT", -8: "BUDGET"}

PARAM_NAMES = ("DT", "DU", "V0", "MASS", "CL_CD", "G", "L0", "D0", "TAU", "TAU_ROLL", "MAX_ROLL_RATE", "MAX_BANK",
               "V_MIN", "V_MAX", "N_C", "R_MAX", "RADIUS_LERP", "R_H", "SIGMA", "W_SEP", "W_ALIGN", "W_COH",
               "BLIND_COS", "W_ROOST_V", "H_ROOST_V", "Z0", "GRID_CELL", "RADIUS_EXP")


class FlockError(RuntimeError):
    """A C-ABI call returned an error status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"FLK_ERR_{ERRORS.get(code, code)} ({code}): {msg}")
        self.code = code


class PassTimes(C.Structure):
    _fields_ = [("hash_ms", C.c_double), ("scan_ms", C.c_double), ("sort_ms", C.c_double),
                ("decide_ms", C.c_double), ("integrate_ms", C.c_double), ("total_ms", C.c_double),
                ("timed_steps", C.c_int32)]


class PoolStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("rejected", C.c_uint64),
                ("bird_steps", C.c_uint64), ("resident_bytes", C.c_uint64), ("chunks", C.c_uint64),
                ("busy_ms", C.c_double)]


_lib: Optional[C.CDLL] = None
_P = C.c_void_p
_PF = C.POINTER(C.c_float)
_PU = C.POINTER(C.c_uint32)
_PI = C.POINTER(C.c_int32)
_PU64 = C.POINTER(C.c_uint64)
_PD = C.POINTER(C.c_double)

_SIGS = {
    "flk_open_host": (C.c_int, [C.c_int32, C.c_uint32, C.c_float, _PF, C.POINTER(_P)]),
    "flk_open_file": (C.c_int, [C.c_int32, C.c_char_p, C.POINTER(_P)]),
    "flk_step": (C.c_int, [_P, C.c_uint32]),
    "flk_step_timed": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.POINTER(PassTimes)]),
    "flk_read_host": (C.c_int, [_P, _PF, _PF]),
    "flk_write_file": (C.c_int, [_P, C.c_char_p]),
    "flk_size": (C.c_int, [_P, _PU, _PU]),
    "flk_decide_occupancy": (C.c_int, [_P, C.c_uint64, _PI, _PI, _PI, _PU64]),
    "flk_device_error_text": (C.c_char_p, [C.c_uint32]),
    "flk_debug_scan_timeout": (C.c_int, [_P, C.c_uint32, C.c_uint32]),
    "flk_step_debug": (C.c_int, [_P, _PU, _PU, _PU, _PU]),
    "flk_counters": (C.c_int, [_P, _PU64, _PU64, _PU64]),
    "flk_step_f64": (C.c_int, [_P, _PD, _PD]),
    "flk_time_steps": (C.c_int, [_P, C.c_uint32, C.c_uint64, _PF]),
    "flk_close": (None, [_P]),
    "flk_batch_create": (C.c_int, [C.c_int32, C.POINTER(_P)]),
    "flk_batch_add": (C.c_int, [_P, C.c_uint32, C.c_float, _PF, _PI]),
    "flk_batch_remove": (C.c_int, [_P, C.c_int32]),
    "flk_batch_step": (C.c_int, [_P, C.c_uint32]),
    "flk_batch_step_each": (C.c_int, [_P, _PI, _PU, C.c_uint32]),
    "flk_batch_read": (C.c_int, [_P, C.c_int32, _PF, _PF]),
    "flk_batch_step_debug": (C.c_int, [_P, _PI, C.c_uint32, _PU, _PU, _PU, _PU]),
    "flk_batch_step_f64": (C.c_int, [_P, _PI, C.c_uint32, _PD, _PD]),
    "flk_batch_graph_counts": (C.c_int, [_P, _PU64, _PU64]),
    "flk_batch_tune": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "flk_batch_tune_cell": (C.c_int, [_P, C.c_float]),
    "flk_tune_cell": (C.c_int, [_P, C.c_float]),
    "flk_batch_tune_decide": (C.c_int, [_P, C.c_int32]),
    "flk_tune_decide": (C.c_int, [_P, C.c_int32]),
    "flk_batch_counters": (C.c_int, [_P, _PU64, _PU64, _PU64]),
    "flk_batch_time_steps": (C.c_int, [_P, C.c_uint32, _PD]),
    "flk_batch_step_timed": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.POINTER(PassTimes)]),
    "flk_batch_destroy": (None, [_P]),
    "flk_pool_create": (C.c_int, [C.c_int32, C.c_uint64, C.c_uint32, C.POINTER(_P)]),
    "flk_pool_submit": (C.c_int, [_P, C.c_uint32, C.c_float, _PF, C.c_uint32, _PF, _PF, _PU64]),
    "flk_pool_submit_file": (C.c_int, [_P, C.c_char_p, C.c_uint32, _PF, C.c_uint32, _PF, _PU64, _PU]),
    "flk_pool_snapshot": (C.c_int, [_P, C.c_uint64, _PF, _PF, _PU, C.c_char_p]),
    "flk_pool_error_report": (C.c_int, [_P, C.c_uint64, _PD, _PD, _PU]),
    "flk_pool_poll": (C.c_int, [_P, C.c_uint64, _PI]),
    "flk_pool_wait": (C.c_int, [_P, C.c_uint64, _PD]),
    "flk_pool_stats_get": (C.c_int, [_P, C.POINTER(PoolStats)]),
    "flk_pool_destroy": (None, [_P]),
    "flk_last_error": (C.c_char_p, []),
    "flk_buckets_for": (C.c_uint32, [C.c_uint32]),
    "flk_file_info": (C.c_int, [C.c_char_p, _PU, _PF]),
    "flk_generate": (C.c_int, [C.c_uint32, C.c_uint64, _PF]),
    "flk_params": (C.c_int, [_PF, C.c_int32]),
    "flk_bytes_for": (C.c_uint64, [C.c_uint32]),
    "flk_kernels_per_step": (C.c_int, []),
    "flk_pin": (C.c_int, [C.c_void_p, C.c_uint64]),
    "flk_unpin": (C.c_int, [C.c_void_p]),
}


def lib() -> C.CDLL:
    """Loads the in-tree native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"native library missing: {LIB_PATH}; run python -m murmuration_kernels_gb300.build")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def header_symbols() -> list[str]:
    """Function names declared in include/flock_gb300.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(flk_[a-z0-9_]+)\s*\(", text)))


def _check(rc: int) -> None:
    if rc != FLK_OK:
        raise FlockError(rc, lib().flk_last_error().decode(errors="replace"))


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(_PF)


def _uptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(_PU)


def _words(words: np.ndarray) -> np.ndarray:
    w = np.ascontiguousarray(words, dtype=np.float32)
    if w.ndim != 2 or w.shape[1] != WORDS:
        w = w.reshape(-1, WORDS)
    return w


# ---- format helpers (state.rs:104-171) --------------------------------------
def read_flk(path: str) -> tuple[float, np.ndarray]:
    """Returns (time, words[n, 15] float32) of a FLK1 file."""
    raw = open(path, "rb").read()
    if len(raw) < 16 or raw[:4] != b"FLK1":
        raise ValueError(f"{path}: not a FLK1 file")
    n, words = np.frombuffer(raw[4:12], dtype="<u4")
    if words != WORDS:
        raise ValueError(f"{path}: unexpected words per bird")
    time = float(np.frombuffer(raw[12:16], dtype="<f4")[0])
    body = np.frombuffer(raw[16:16 + int(n) * WORDS * 4], dtype="<f4")
    if body.size != int(n) * WORDS:
        raise ValueError(f"{path}: truncated")
    return time, body.reshape(int(n), WORDS).copy()


def write_flk(path: str, time: float, words: np.ndarray) -> None:
    w = _words(words)
    head = np.array([0x314B4C46, w.shape[0], WORDS], dtype="<u4").tobytes() + np.float32(time).astype("<f4").tobytes()
    with open(path, "wb") as f:
        f.write(head)
        f.write(w.astype("<f4").tobytes())


def generate(n: int, seed: int = 1) -> np.ndarray:
    """The benchmark scatter (state.rs:79-101): words[n, 15] at time 0."""
    w = np.zeros((n, WORDS), dtype=np.float32)
    _check(lib().flk_generate(n, seed, _fptr(w)))
    return w


def file_info(path: str) -> tuple[int, float]:
    """(birds, time) from a .flk header, read by the library."""
    n = C.c_uint32()
    t = C.c_float()
    _check(lib().flk_file_info(path.encode(), C.byref(n), C.byref(t)))
    return n.value, t.value


def device_error_text(word: int) -> str:
    """What a device error word means (the text FLK_ERR_DEVICE reports)."""
    return lib().flk_device_error_text(word).decode()


def buckets_for(n: int) -> int:
    return int(lib().flk_buckets_for(n))


def params() -> dict[str, float]:
    out = np.zeros(len(PARAM_NAMES), dtype=np.float32)
    k = lib().flk_params(_fptr(out), len(PARAM_NAMES))
    return dict(zip(PARAM_NAMES[:k], out[:k].tolist()))


def bytes_for(n: int) -> int:
    return int(lib().flk_bytes_for(n))


def kernels_per_step() -> int:
    return int(lib().flk_kernels_per_step())


class pinned:
    """Context manager that page-locks numpy arrays for the duration."""

    def __init__(self, *arrays: np.ndarray):
        self.arrays = [a for a in arrays if a.nbytes]

    def __enter__(self):
        for a in self.arrays:
            _check(lib().flk_pin(a.ctypes.data, a.nbytes))
        return self

    def __exit__(self, *exc):
        for a in self.arrays:
            lib().flk_unpin(a.ctypes.data)


def neighbours(words: np.ndarray) -> np.ndarray:
    """The u32 neighbour-count column of a words array."""
    return _words(words)[:, 13].view(np.uint32)


# ---- plain single flock ------------------------------------------------------
class Flock:
    """One resident flock (the drop-in for one `flock_cuda` run)."""

    def __init__(self, words: np.ndarray, time: float = 0.0, device: int = -1):
        w = _words(words)
        self.n = w.shape[0]
        self._h = _P()
        _check(lib().flk_open_host(device, self.n, C.c_float(time), _fptr(w), C.byref(self._h)))
        nb = C.c_uint32()
        _check(lib().flk_size(self._h, None, C.byref(nb)))
        self.buckets = nb.value

    @classmethod
    def open(cls, path: str, device: int = -1) -> "Flock":
        """Reads and uploads a .flk file through the C ABI (flk_open_file)."""
        self = cls.__new__(cls)
        self._h = _P()
        _check(lib().flk_open_file(device, path.encode(), C.byref(self._h)))
        n, nb = C.c_uint32(), C.c_uint32()
        _check(lib().flk_size(self._h, C.byref(n), C.byref(nb)))
        self.n, self.buckets = n.value, nb.value
        return self

    def step(self, steps: int = 1) -> None:
        _check(lib().flk_step(self._h, steps))

    def step_timed(self, steps: int, warmup: int = 0) -> dict[str, float]:
        pt = PassTimes()
        _check(lib().flk_step_timed(self._h, steps, warmup, C.byref(pt)))
        return {k: getattr(pt, k) for k, _ in PassTimes._fields_}

    def read(self, out: Optional[np.ndarray] = None) -> tuple[float, np.ndarray]:
        w = out if out is not None else np.empty((self.n, WORDS), dtype=np.float32)
        t = C.c_float()
        _check(lib().flk_read_host(self._h, C.byref(t), _fptr(w)))
        return float(t.value), w

    def write(self, path: str) -> None:
        _check(lib().flk_write_file(self._h, path.encode()))

    def step_debug(self) -> dict[str, np.ndarray]:
        """One step; returns keys[n], offsets[B+1], sorted[n], sets[n, 8]."""
        keys = np.zeros(self.n, dtype=np.uint32)
        offs = np.zeros(self.buckets + 1, dtype=np.uint32)
        srt = np.zeros(self.n, dtype=np.uint32)
        sets = np.zeros((self.n, 8), dtype=np.uint32)
        _check(lib().flk_step_debug(self._h, _uptr(keys), _uptr(offs), _uptr(srt), _uptr(sets)))
        return {"keys": keys, "offsets": offs, "sorted": srt, "sets": sets}

    def step_f64(self) -> tuple[np.ndarray, dict[str, float]]:
        """One step (as step(1)) that also evaluates it in FP64 from the same
        state: (FP64 post-step state [n, 15], error report of the f32 step)."""
        out = np.empty((self.n, WORDS), dtype=np.float64)
        rep = np.zeros(4, dtype=np.float64)
        _check(lib().flk_step_f64(self._h, out.ctypes.data_as(_PD), rep.ctypes.data_as(_PD)))
        return out, _f64_report(rep)

    def counters(self) -> tuple[int, int, int]:
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(lib().flk_counters(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def decide_occupancy(self, extra_smem: int = 0) -> dict[str, int]:
        """Reserves `extra_smem` more bytes of shared memory per decide CTA (the
        reference's --decide-smem) and returns decide's launch occupancy."""
        bps, th, tpsm, sm = C.c_int32(), C.c_int32(), C.c_int32(), C.c_uint64()
        _check(lib().flk_decide_occupancy(self._h, extra_smem, C.byref(bps), C.byref(th), C.byref(tpsm),
                                          C.byref(sm)))
        return {"blocks_per_sm": bps.value, "threads": th.value, "threads_per_sm": tpsm.value,
                "smem_bytes": sm.value}

    def tune_cell(self, cell: float) -> None:
        """The production cell edge in m (steps without grid output)."""
        _check(lib().flk_tune_cell(self._h, C.c_float(cell)))

    def tune_decide(self, staged: int) -> None:
        """The production decide kernel: 0 sweeps the state, 1 stages cells in shared memory."""
        _check(lib().flk_tune_decide(self._h, staged))

    def debug_scan_timeout(self, skip_tile: int = 0, spin_limit: int = 1000) -> None:
        """Test hook: the next step_debug's scan gives up waiting (FLK_ERR_DEVICE)."""
        _check(lib().flk_debug_scan_timeout(self._h, skip_tile, spin_limit))

    def time_steps(self, steps: int, flush_bytes: int = 256 << 20) -> np.ndarray:
        """Device ms of each of `steps` single-step launches, L2 flushed before each.
        Each step counts the next step's grid as in step(); one untimed step
        follows the last, so the flock advances steps + 1."""
        ms = np.zeros(steps, dtype=np.float32)
        _check(lib().flk_time_steps(self._h, steps, flush_bytes, _fptr(ms)))
        return ms

    def close(self) -> None:
        if self._h:
            lib().flk_close(self._h)
            self._h = _P()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- batched -----------------------------------------------------------------
def _f64_report(rep: np.ndarray) -> dict[str, float]:
    return {"max_rel_pos": float(rep[0]), "max_rel_vel": float(rep[1]),
            "neighbour_mismatches": int(rep[2]), "deciding": int(rep[3])}


class Batch:
    """Many independent flocks advanced together (one launch per pass)."""

    def __init__(self, device: int = -1):
        self._h = _P()
        _check(lib().flk_batch_create(device, C.byref(self._h)))
        self.sizes: dict[int, int] = {}

    def add(self, words: np.ndarray, time: float = 0.0) -> int:
        w = _words(words)
        i = C.c_int32()
        _check(lib().flk_batch_add(self._h, w.shape[0], C.c_float(time), _fptr(w), C.byref(i)))
        self.sizes[i.value] = w.shape[0]
        return i.value

    def remove(self, fid: int) -> None:
        _check(lib().flk_batch_remove(self._h, fid))
        self.sizes.pop(fid, None)

    def step(self, steps: int = 1) -> None:
        _check(lib().flk_batch_step(self._h, steps))

    def step_each(self, ids: Sequence[int], steps: Sequence[int]) -> None:
        a = np.asarray(ids, dtype=np.int32)
        s = np.asarray(steps, dtype=np.uint32)
        _check(lib().flk_batch_step_each(self._h, a.ctypes.data_as(_PI), _uptr(s), len(a)))

    def read(self, fid: int) -> tuple[float, np.ndarray]:
        w = np.empty((self.sizes[fid], WORDS), dtype=np.float32)
        t = C.c_float()
        _check(lib().flk_batch_read(self._h, fid, C.byref(t), _fptr(w)))
        return float(t.value), w

    def step_debug(self, ids: Sequence[int]) -> list[dict[str, np.ndarray]]:
        a = np.asarray(ids, dtype=np.int32)
        ns = [self.sizes[i] for i in ids]
        bs = [buckets_for(n) for n in ns]
        keys = np.zeros(sum(ns), dtype=np.uint32)
        offs = np.zeros(sum(b + 1 for b in bs), dtype=np.uint32)
        srt = np.zeros(sum(ns), dtype=np.uint32)
        sets = np.zeros((sum(ns), 8), dtype=np.uint32)
        _check(lib().flk_batch_step_debug(self._h, a.ctypes.data_as(_PI), len(a), _uptr(keys), _uptr(offs),
                                          _uptr(srt), _uptr(sets)))
        out, k, o = [], 0, 0
        for n, b in zip(ns, bs):
            out.append({"keys": keys[k:k + n], "offsets": offs[o:o + b + 1], "sorted": srt[k:k + n],
                        "sets": sets[k:k + n]})
            k += n
            o += b + 1
        return out

    def step_f64(self, ids: Sequence[int]) -> list[tuple[np.ndarray, dict[str, float]]]:
        """One step of each listed flock with its FP64 evaluation (as
        Flock.step_f64): per id (FP64 post-step state [n, 15], error report)."""
        a = np.asarray(ids, dtype=np.int32)
        ns = [self.sizes[i] for i in ids]
        out = np.empty((sum(ns), WORDS), dtype=np.float64)
        rep = np.zeros((len(a), 4), dtype=np.float64)
        _check(lib().flk_batch_step_f64(self._h, a.ctypes.data_as(_PI), len(a), out.ctypes.data_as(_PD),
                                        rep.ctypes.data_as(_PD)))
        res, k = [], 0
        for i, n in enumerate(ns):
            res.append((out[k:k + n], _f64_report(rep[i])))
            k += n
        return res

    def graph_counts(self) -> tuple[int, int]:
        """(chunk graphs instantiated, chunk graphs updated in place) so far."""
        a, b = C.c_uint64(), C.c_uint64()
        _check(lib().flk_batch_graph_counts(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def tune(self, stream_bps: int = 0, decide_bps: int = 0, decide_threads: int = 0, graph_chunk: int = 0,
             cell: float = 0.0, staged: int = -1) -> None:
        """Launch shapes, the production cell edge in m (0 keeps a value) and
        the decide kernel (0 direct, 1 staged; -1 keeps it)."""
        _check(lib().flk_batch_tune(self._h, stream_bps, decide_bps, decide_threads, graph_chunk))
        if cell:
            _check(lib().flk_batch_tune_cell(self._h, C.c_float(cell)))
        if staged >= 0:
            _check(lib().flk_batch_tune_decide(self._h, staged))

    def time_steps(self, steps: int) -> float:
        ms = C.c_double()
        _check(lib().flk_batch_time_steps(self._h, steps, C.byref(ms)))
        return ms.value

    def step_timed(self, steps: int, warmup: int = 0) -> dict[str, float]:
        pt = PassTimes()
        _check(lib().flk_batch_step_timed(self._h, steps, warmup, C.byref(pt)))
        return {k: getattr(pt, k) for k, _ in PassTimes._fields_}

    def counters(self) -> tuple[int, int, int]:
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(lib().flk_batch_counters(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def close(self) -> None:
        if self._h:
            lib().flk_batch_destroy(self._h)
            self._h = _P()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- served ------------------------------------------------------------------
class Pool:
    """Continuous batching of simulate(flock, steps) requests on one GPU."""

    def __init__(self, budget_bytes: int, chunk_steps: int = 10, device: int = -1):
        self._h = _P()
        _check(lib().flk_pool_create(device, budget_bytes, chunk_steps, C.byref(self._h)))
        self._keep: dict[int, tuple] = {}

    def submit(self, words: np.ndarray, steps: int, time: float = 0.0,
               out: Optional[np.ndarray] = None) -> int:
        w = _words(words)
        o = out if out is not None else np.empty_like(w)
        t = np.zeros(1, dtype=np.float32)
        tk = C.c_uint64()
        _check(lib().flk_pool_submit(self._h, w.shape[0], C.c_float(time), _fptr(w), steps, _fptr(o), _fptr(t),
                                     C.byref(tk)))
        self._keep[tk.value] = (w, o, t)  # buffers must outlive the request
        return tk.value

    def submit_file(self, path: str, steps: int) -> int:
        """simulate(flock, steps) for the state in a .flk file (the pool keeps its own copy)."""
        n, _ = file_info(path)
        o = np.empty((n, WORDS), dtype=np.float32)
        t = np.zeros(1, dtype=np.float32)
        tk = C.c_uint64()
        got = C.c_uint32()
        _check(lib().flk_pool_submit_file(self._h, path.encode(), steps, _fptr(o), n, _fptr(t), C.byref(tk),
                                          C.byref(got)))
        self._keep[tk.value] = (None, o, t)
        return tk.value

    def snapshot(self, ticket: int, path: Optional[str] = None) -> tuple[float, np.ndarray, int]:
        """The request's current state without pausing the other flocks:
        (time, words, steps done); with `path`, also written as a .flk file."""
        if ticket not in self._keep:
            raise ValueError("snapshot: unknown ticket, or its result was already collected by wait()")
        o = self._keep[ticket][1]
        w = np.empty_like(o)
        t = np.zeros(1, dtype=np.float32)
        k = C.c_uint32()
        _check(lib().flk_pool_snapshot(self._h, ticket, _fptr(w), _fptr(t), C.byref(k),
                                       path.encode() if path else None))
        return float(t[0]), w, k.value

    def error_report(self, ticket: int) -> tuple[np.ndarray, dict[str, float], int]:
        """The FP64 evaluation of the request's next step, run on a copy of its
        current state (the served flock is not advanced): (FP64 post-step
        state [n, 15], error report, steps done at the snapshot)."""
        if ticket not in self._keep:
            raise ValueError("error_report: unknown ticket, or its result was already collected by wait()")
        n = self._keep[ticket][1].shape[0]
        out = np.empty((n, WORDS), dtype=np.float64)
        rep = np.zeros(4, dtype=np.float64)
        k = C.c_uint32()
        _check(lib().flk_pool_error_report(self._h, ticket, out.ctypes.data_as(_PD), rep.ctypes.data_as(_PD),
                                           C.byref(k)))
        return out, _f64_report(rep), k.value

    def poll(self, ticket: int) -> int:
        s = C.c_int32()
        _check(lib().flk_pool_poll(self._h, ticket, C.byref(s)))
        return s.value

    def wait(self, ticket: int) -> tuple[float, np.ndarray, float]:
        """Blocks; returns (time, words, latency_ms)."""
        lat = C.c_double()
        _check(lib().flk_pool_wait(self._h, ticket, C.byref(lat)))
        _, o, t = self._keep.pop(ticket)
        return float(t[0]), o, lat.value

    def stats(self) -> dict[str, float]:
        s = PoolStats()
        _check(lib().flk_pool_stats_get(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in PoolStats._fields_}

    def close(self) -> None:
        if self._h:
            lib().flk_pool_destroy(self._h)
            self._h = _P()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
