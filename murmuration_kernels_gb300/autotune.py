"""Launch-shape and cell-size autotuner for the flock engine.

The engine's passes are persistent grid-stride kernels whose shapes are
runtime parameters: CTAs per SM of the streaming passes (hash/count,
scatter, integrate), `decide`'s CTA size and CTAs per SM, and the number of
steps captured per CUDA graph. The production steps' cell edge is one too
(`cell`, in metres; cells are sorted in quarter-cell z-slabs): a smaller cell
means fewer candidates per deciding bird but more cells per search box (a
box of more than 32 cells leaves decide's fast path) and shorter runs for the
sort. Any edge finds the same neighbours. Clusters are not used, so there is
no cluster shape to tune. The best values depend on the workload (one
1M-bird flock vs hundreds of small flocks), so the tuner measures them on the
actual batch: coordinate descent over each knob's candidate values, each
candidate timed with CUDA events over a few graph-launched steps, keeping a
change only when it beats the incumbent by more than the noise margin.

Results are cached per (GPU name, workload signature) in a JSON file so a
served or batched run can reuse them:

    from murmuration_kernels_gb300 import autotune
    shape = autotune.tune(batch, steps=10)      # applies and returns the best shape
"""
from __future__ import annotations

import json
import os
from typing import Optional

SPACE = {
    "cell": [3.5, 3.75, 4.0, 4.5],
    "stream_bps": [4, 8, 16],
    "decide_bps": [1, 2, 4, 8],
    "decide_threads": [256, 512, 1024],
    "graph_chunk": [5, 10, 20],
}
DEFAULT = {"cell": 4.0, "stream_bps": 8, "decide_bps": 1, "decide_threads": 1024, "graph_chunk": 10}
CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")


def _signature(batch) -> str:
    sizes = sorted(batch.sizes.values())
    total = sum(sizes)
    # flocks bucketed by size decade: shapes that work for one mix work for similar ones
    hist = {}
    for n in sizes:
        d = len(str(max(n, 1)))
        hist[d] = hist.get(d, 0) + 1
    return f"birds={total // 100_000 * 100_000}|flocks={len(sizes)}|" + ",".join(f"{k}:{v}" for k, v in sorted(hist.items()))


def _apply(batch, shape: dict) -> None:
    batch.tune(stream_bps=shape["stream_bps"], decide_bps=shape["decide_bps"],
               decide_threads=shape["decide_threads"], graph_chunk=shape["graph_chunk"], cell=shape["cell"])


def _time(batch, shape: dict, steps: int, reps: int) -> float:
    _apply(batch, shape)
    batch.time_steps(shape["graph_chunk"])  # capture + warm
    best = float("inf")
    for _ in range(reps):
        best = min(best, batch.time_steps(steps))
    return best / steps


def _load_cache() -> dict:
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def tune(batch, steps: int = 10, reps: int = 2, margin: float = 0.01, gpu: str = "gpu",
         use_cache: bool = True) -> dict:
    """Finds, applies and returns the fastest launch shape for `batch`.

    Every timed candidate advances the batch's flocks (the tuner runs real
    steps), so tune on a copy of the state you care about, or accept the
    extra steps. Returns {"shape": {...}, "ms_per_step": t, "trials": k}."""
    key = f"{gpu}|{_signature(batch)}"
    cache = _load_cache() if use_cache else {}
    if key in cache:
        _apply(batch, cache[key]["shape"])
        return dict(cache[key], cached=True)
    best = dict(DEFAULT)
    best_t = _time(batch, best, steps, reps)
    trials = 1
    for knob, values in SPACE.items():
        start = best[knob]  # timed already, as part of the incumbent
        for v in values:
            if v == start or v == best[knob]:
                continue
            cand = dict(best, **{knob: v})
            t = _time(batch, cand, steps, reps)
            trials += 1
            if t < best_t * (1.0 - margin):
                best, best_t = cand, t
    _apply(batch, best)
    result = {"shape": best, "ms_per_step": best_t, "trials": trials}
    if use_cache:
        cache[key] = result
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        with open(CACHE, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
    return dict(result, cached=False)


def cached(batch, gpu: str = "gpu") -> Optional[dict]:
    return _load_cache().get(f"{gpu}|{_signature(batch)}")
