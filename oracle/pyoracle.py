"""ctypes wrapper of the CPU oracle (oracle/flock_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's CPU-baseline / reference arm. The product
package never imports it.

Bird records are numpy float32 arrays of shape (n, 15) in .flk word order;
the neighbour count (word 13) is u32 bits.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
CLI = os.path.join(HERE, "_build", "flock_ref_c")
WORDS = 15

_lib: Optional[C.CDLL] = None
_PF = C.POINTER(C.c_float)
_PU = C.POINTER(C.c_uint32)
_PD = C.POINTER(C.c_double)
_PB = C.POINTER(C.c_uint8)


def build() -> None:
    """Compiles the oracle with its Makefile (gcc, -ffp-contract=off)."""
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or not os.path.exists(CLI):
            build()
        L = C.CDLL(LIB)
        sig = {
            "orc_params": (None, [_PF]),
            "orc_param_name": (C.c_char_p, [C.c_int]),
            "orc_set_mix": (C.c_uint32, [C.c_uint32]),
            "orc_radius_step": (C.c_float, [C.c_float, C.c_uint32]),
            "orc_scatter": (None, [C.c_uint32, C.c_uint64, _PF]),
            "orc_step": (C.c_float, [_PF, C.c_uint32, C.c_float, _PU, _PB, C.c_int]),
            "orc_step_f64": (C.c_double, [_PF, C.c_uint32, C.c_float, _PD, C.c_int]),
            "orc_decide_sample": (C.c_double, [_PF, C.c_uint32, _PU, C.c_uint32, C.c_int]),
            "orc_integrate_all": (None, [_PF, C.c_uint32, C.c_int]),
            "orc_step_grid": (C.c_float, [_PF, C.c_uint32, C.c_float, C.c_int]),
            "orc_decide_many": (None, [_PF, C.c_uint32, _PU, C.c_uint32, _PU, _PF, C.c_int]),
            "orc_buckets_for": (C.c_uint32, [C.c_uint32]),
            "orc_grid": (None, [_PF, C.c_uint32, C.c_uint32, _PU, _PU, _PU]),
            "orc_check_grid": (C.c_int, [_PU, _PU, _PU, C.c_uint32, C.c_uint32, _PF]),
            "orc_stats": (None, [_PF, C.c_uint32, _PF]),
            "orc_diff": (C.c_int, [_PF, _PF, C.c_uint32, C.c_float, C.c_float, C.c_uint32, C.c_float, _PF, _PU, _PU]),
            "orc_statdiff": (C.c_int, [_PF, _PF, C.c_uint32, _PF]),
            "orc_max_threads": (C.c_int, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _w(words: np.ndarray) -> np.ndarray:
    w = np.ascontiguousarray(words, dtype=np.float32)
    return w.reshape(-1, WORDS)


def _f(a):
    return a.ctypes.data_as(_PF)


def _u(a):
    return None if a is None else a.ctypes.data_as(_PU)


def params() -> dict[str, float]:
    out = np.zeros(28, dtype=np.float32)
    lib().orc_params(_f(out))
    return {lib().orc_param_name(k).decode(): float(out[k]) for k in range(28)}


def params_raw() -> np.ndarray:
    out = np.zeros(28, dtype=np.float32)
    lib().orc_params(_f(out))
    return out


def set_mix(j: int) -> int:
    return int(lib().orc_set_mix(j))


def radius_step(r: float, n: int) -> float:
    return float(lib().orc_radius_step(C.c_float(r), n))


def scatter(n: int, seed: int = 1) -> np.ndarray:
    out = np.zeros((n, WORDS), dtype=np.float32)
    lib().orc_scatter(n, seed, _f(out))
    return out


def step(words: np.ndarray, time: float, threads: int = 0, with_sets: bool = True):
    """One oracle step (model.rs:182-200). Returns (time, words, sets[n,8], due[n])."""
    w = _w(words).copy()
    n = w.shape[0]
    sets = np.zeros((n, 8), dtype=np.uint32) if with_sets else None
    due = np.zeros(n, dtype=np.uint8)
    t = lib().orc_step(_f(w), n, C.c_float(time), _u(sets), due.ctypes.data_as(_PB), threads)
    return float(np.float32(t)), w, sets, due.astype(bool)


def steps(words: np.ndarray, time: float, k: int, threads: int = 0):
    w = _w(words).copy()
    n = w.shape[0]
    t = C.c_float(time)
    for _ in range(k):
        t = C.c_float(lib().orc_step(_f(w), n, t, None, None, threads))
    return float(t.value), w


def step_f64(words: np.ndarray, time: float, threads: int = 0) -> np.ndarray:
    """FP64 evaluation of one step from the same f32 input: (n, 15) float64."""
    w = _w(words)
    out = np.zeros((w.shape[0], WORDS), dtype=np.float64)
    lib().orc_step_f64(_f(w), w.shape[0], C.c_float(time), out.ctypes.data_as(_PD), threads)
    return out


def decide_sample(words: np.ndarray, idx: np.ndarray, threads: int = 0) -> float:
    w = _w(words)
    i = np.ascontiguousarray(idx, dtype=np.uint32)
    return float(lib().orc_decide_sample(_f(w), w.shape[0], _u(i), len(i), threads))


def decide_many(words: np.ndarray, idx: np.ndarray, threads: int = 0):
    """decide() for the listed birds: (sets[m, 8] u32, decisions[m, 6] f32 =
    force xyz, radius, neighbours (u32 bits), centrality)."""
    w = _w(words)
    i = np.ascontiguousarray(idx, dtype=np.uint32)
    sets = np.zeros((len(i), 8), dtype=np.uint32)
    dec = np.zeros((len(i), 6), dtype=np.float32)
    lib().orc_decide_many(_f(w), w.shape[0], _u(i), len(i), _u(sets), _f(dec), threads)
    return sets, dec


def integrate_all(words: np.ndarray, threads: int = 0) -> np.ndarray:
    w = _w(words).copy()
    lib().orc_integrate_all(_f(w), w.shape[0], threads)
    return w


def step_grid(words: np.ndarray, time: float, threads: int = 0):
    """One step with the reference GPU backend's grid algorithm on host cores
    (cuda/flock.cu:190-290): the CPU grid baseline. Returns (time, words)."""
    w = _w(words).copy()
    t = lib().orc_step_grid(_f(w), w.shape[0], time, threads)
    return t, w


def buckets_for(n: int) -> int:
    return int(lib().orc_buckets_for(n))


def grid(words: np.ndarray, buckets: Optional[int] = None):
    """Canonical grid: keys[n], offsets[B+1], sorted[n] in (bucket, bird) order."""
    w = _w(words)
    n = w.shape[0]
    b = buckets or buckets_for(n)
    keys = np.zeros(n, dtype=np.uint32)
    offs = np.zeros(b + 1, dtype=np.uint32)
    srt = np.zeros(n, dtype=np.uint32)
    lib().orc_grid(_f(w), n, b, _u(keys), _u(offs), _u(srt))
    return keys, offs, srt


def check_grid(keys, offsets, sorted_, buckets: int, words: Optional[np.ndarray] = None) -> int:
    k = np.ascontiguousarray(keys, dtype=np.uint32)
    o = np.ascontiguousarray(offsets, dtype=np.uint32)
    s = np.ascontiguousarray(sorted_, dtype=np.uint32)
    w = None if words is None else _w(words)
    return int(lib().orc_check_grid(_u(k), _u(o), _u(s), len(k), buckets, None if w is None else _f(w)))


def stats(words: np.ndarray) -> np.ndarray:
    out = np.zeros(4, dtype=np.float32)
    w = _w(words)
    lib().orc_stats(_f(w), w.shape[0], _f(out))
    return out


def diff(a: np.ndarray, b: np.ndarray, pos_tol=1e-3, vel_tol=1e-3, allow=0, outlier_max=1e-2):
    """main.rs:136-208. Returns (ok, maxes[7], mismatches, outliers)."""
    x, y = _w(a), _w(b)
    out = np.zeros(7, dtype=np.float32)
    mm, ol = C.c_uint32(), C.c_uint32()
    ok = lib().orc_diff(_f(x), _f(y), x.shape[0], pos_tol, vel_tol, allow, outlier_max, _f(out), C.byref(mm),
                        C.byref(ol))
    return bool(ok), out, mm.value, ol.value


def statdiff(a: np.ndarray, b: np.ndarray):
    x, y = _w(a), _w(b)
    out = np.zeros(4, dtype=np.float32)
    ok = lib().orc_statdiff(_f(x), _f(y), x.shape[0], _f(out))
    return bool(ok), out


def max_threads() -> int:
    return int(lib().orc_max_threads())
