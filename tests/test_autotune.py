"""The launch-shape autotuner's host logic (coordinate descent, noise margin,
cache), driven by a fake batch whose step time is a known function of the
shape. No GPU."""
from __future__ import annotations

import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _autotune():
    # the module needs no native library; load it without importing the package
    spec = importlib.util.spec_from_file_location("flk_autotune",
                                                  os.path.join(ROOT, "murmuration_kernels_gb300", "autotune.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class FakeBatch:
    """time_steps(k) returns k * cost(shape) for the shape last applied."""

    def __init__(self, cost, sizes=(1000, 20000, 300000)):
        self.cost = cost
        self.sizes = {i: n for i, n in enumerate(sizes)}
        self.shape = None
        self.applied = []

    def tune(self, stream_bps, decide_bps, decide_threads, graph_chunk, cell):
        self.shape = dict(stream_bps=stream_bps, decide_bps=decide_bps, decide_threads=decide_threads,
                          graph_chunk=graph_chunk, cell=cell)
        self.applied.append(dict(self.shape))

    def time_steps(self, k):
        return k * self.cost(self.shape)


def test_descent_finds_the_fastest_shape_one_knob_at_a_time(tmp_path, monkeypatch):
    at = _autotune()
    monkeypatch.setattr(at, "CACHE", str(tmp_path / "autotune.json"))
    best = {"stream_bps": 16, "decide_bps": 2, "decide_threads": 512, "graph_chunk": 20, "cell": 3.5}
    # separable cost: each knob away from its best value adds time
    cost = lambda s: 1.0 + sum(0.1 * (s[k] != best[k]) for k in best)
    b = FakeBatch(cost)
    r = at.tune(b, steps=10, use_cache=False)
    assert r["shape"] == best and b.shape == best
    assert r["ms_per_step"] == pytest.approx(1.0)
    # the default, then every other value of every knob once
    assert r["trials"] == 1 + sum(len(v) - 1 for v in at.SPACE.values())


def test_changes_within_the_noise_margin_are_not_taken(tmp_path, monkeypatch):
    at = _autotune()
    monkeypatch.setattr(at, "CACHE", str(tmp_path / "autotune.json"))
    # every other shape is 0.5 % faster than the default: below the 1 % margin
    cost = lambda s: 1.0 if s == at.DEFAULT else 0.995
    b = FakeBatch(cost)
    r = at.tune(b, steps=10, use_cache=False)
    assert r["shape"] == at.DEFAULT


def test_cache_round_trip_and_signature(tmp_path, monkeypatch):
    at = _autotune()
    monkeypatch.setattr(at, "CACHE", str(tmp_path / "autotune.json"))
    best = {"stream_bps": 4, "decide_bps": 1, "decide_threads": 1024, "graph_chunk": 5, "cell": 4.0}
    cost = lambda s: 1.0 + sum(0.1 * (s[k] != best[k]) for k in best)
    b = FakeBatch(cost)
    r1 = at.tune(b, steps=10)
    assert r1["cached"] is False and os.path.exists(at.CACHE)
    # a batch with the same size profile reuses the result without timing anything
    b2 = FakeBatch(lambda s: pytest.fail("a cached shape must not be timed"), sizes=(1100, 21000, 310000))
    r2 = at.tune(b2, steps=10)
    assert r2["cached"] is True and r2["shape"] == best and b2.shape == best
    assert at.cached(b2) is not None
    # another size profile (other decades) is a different signature
    b3 = FakeBatch(cost, sizes=(5, 50))
    assert at.cached(b3) is None


def test_cell_axis_is_searched_first_and_kept_only_when_faster(tmp_path, monkeypatch):
    at = _autotune()
    monkeypatch.setattr(at, "CACHE", str(tmp_path / "autotune.json"))
    assert list(at.SPACE)[0] == "cell" and at.DEFAULT["cell"] == 4.0
    # a 4.5 m cell is 3 % faster for this mix; every other knob is neutral
    cost = lambda s: 0.97 if s["cell"] == 4.5 else 1.0
    b = FakeBatch(cost)
    r = at.tune(b, steps=10, use_cache=False)
    assert r["shape"]["cell"] == 4.5 and b.shape["cell"] == 4.5
    assert {k: v for k, v in r["shape"].items() if k != "cell"} == {k: v for k, v in at.DEFAULT.items() if k != "cell"}
