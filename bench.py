#!/usr/bin/env python3
"""Benchmark of the GB300 flock step: bird-updates/s on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Headline (`value`): the plain single-flock step at 1,000,000 birds (seed 1,
the reference's benchmark scatter), K timed steps after W warm-up steps, each
timed step launched alone (one CUDA graph) after a 256 MB write that flushes
the 129 MB L2, device time from CUDA events on the library's stream.

Also on the same line:
  e2e        the same workload through the C ABI from pinned host buffers
             (upload, K steps, download inside the timed region);
  roofline   step bytes (B_alg per bird-update) / step time vs measured HBM peak;
  batched    256 flocks, sizes log-uniform in [1e3, 2e5] (seed 3), 10-step
             graph chunks, against the same flocks run one at a time;
  served     a Poisson stream of simulate(flock, steps) requests (seed 5)
             through the continuous-batching pool: p50/p99 latency and
             aggregate bird-updates/s, against the same requests served one
             at a time through the plain step;
  cpu_baseline  the brute-force CPU oracle on a bounded sample of the workload.
  cpu_grid   the reference GPU backend's grid algorithm restated for the CPU
             (OpenMP, all host cores), full steps of the same workload.

`--impl reference` times the reference's own CPU step (the C restatement of
its flock-ref oracle; the Rust original cannot be built on this image) on all
host cores, on a bounded sample of the same workload per step.

Multi-GPU (torchrun, one rank per GPU): independent replicas of the plain
workload (a single flock does not shard; flocks would be partitioned across
GPUs with no exchange), barrier + max over ranks, value = all ranks' updates.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "bird-updates/s/GPU plain vs batched-served; p50/p99 request latency"
WORDS = 15
FLUSH_BYTES = 256 << 20
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC = os.path.join(ROOT, "profiles", "traffic_step_1m.txt")


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------
def peak_hbm() -> tuple[float, str]:
    try:
        with open(PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def step_traffic_bytes() -> float | None:
    """DRAM bytes (read + write) of one 1M-bird step from the committed ncu summary."""
    try:
        for line in open(TRAFFIC):
            if line.startswith("step_dram_bytes"):
                return float(line.split("=")[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 10 ms during a region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "10"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            # nvidia-smi takes a moment to start: the region begins once it samples
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < 3.0 and self.proc.poll() is None and os.path.getsize(self.path) == 0:
                time.sleep(0.01)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict | None:
        if not self.proc or not self.path:
            return None
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for _, _, r in rows for k in range(4) if r[k].lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    """torch.distributed only under torchrun (N > 1)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world <= 1:
        return None, 0, 1, 0
    import torch
    import torch.distributed as dist

    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return dist, rank, world, local


def aggregate(dist, local_ms: float, local_units: float) -> tuple[float, float]:
    """Max time over ranks, sum of work over ranks (replicas)."""
    if dist is None:
        return local_ms, local_units
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([local_ms], dtype=torch.float64, device=dev)
    u = torch.tensor([local_units], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def log_uniform_sizes(rng, count, lo, hi):
    return np.rint(np.exp(rng.uniform(math.log(lo), math.log(hi), size=count))).astype(np.int64)


# ---------------------------------------------------------------------------
# CPU reference (brute-force oracle) on a bounded sample
# ---------------------------------------------------------------------------
def cpu_sample(words: np.ndarray, budget_s: float, seed: int = 0) -> dict:
    """Decide for a random sample of deciding birds (brute force over all N) plus
    integrate of all N, extrapolated to one full step; all host threads."""
    from oracle import pyoracle as o

    n = len(words)
    due = np.nonzero(np.float32(0.005) >= words[:, 12])[0]
    threads = o.max_threads()
    rng = np.random.default_rng(seed)
    probe = rng.choice(due, size=min(len(due), max(threads, 16)), replace=False)
    t0 = time.perf_counter()
    o.decide_sample(words, probe)
    per_bird = (time.perf_counter() - t0) / len(probe)
    m = int(min(len(due), max(len(probe), budget_s / max(per_bird, 1e-9))))
    sample = rng.choice(due, size=m, replace=False)
    t0 = time.perf_counter()
    o.decide_sample(words, sample)
    t_dec = time.perf_counter() - t0
    t0 = time.perf_counter()
    o.integrate_all(words)
    t_int = time.perf_counter() - t0
    step_s = t_dec * len(due) / m + t_int
    return {"value": n / step_s, "unit": "bird-updates/s", "cores": threads, "kind": "port",
            "sample": f"brute-force decide of {m} of the {len(due)} deciding birds (each against all {n}) "
                      f"+ integrate of all {n}; extrapolated to one step ({step_s:.3f} s)",
            "sample_wall_s": round(t_dec + t_int, 3), "extrapolated_step_s": step_s}


def cpu_grid_steps(words: np.ndarray, steps: int) -> dict:
    """Full steps of the workload with the reference GPU backend's grid
    algorithm on all host cores (cuda/flock.cu:190-290 restated in the oracle)."""
    from oracle import pyoracle as o

    n = len(words)
    threads = o.max_threads()
    t, w = 0.0, words
    t0 = time.perf_counter()
    for _ in range(steps):
        t, w = o.step_grid(w, t)
    wall = time.perf_counter() - t0
    return {"value": n * steps / wall, "unit": "bird-updates/s", "cores": threads, "kind": "port",
            "sample": f"{steps} full grid steps of {n} birds (cell walks with the exact cell check, as "
                      f"cuda/flock.cu's decide), {wall:.2f} s"}


def workload_config(n: int, seed: int, world: int) -> dict:
    """The `config` of both arms' lines (the same dict, so the arms compare)."""
    return {"workload": f"plain single-flock step, {n:,} birds, seed {seed}", "birds": n, "seed": seed,
            "parallelism": "replicas" if world > 1 else "single GPU",
            "l2": "flushed before every timed step (256 MB write); each step one CUDA-graph launch "
                  "whose integrate counts the next step's grid, as in flk_step's multi-step runs"}


def run_reference(args, dist, rank):
    """The reference's CPU step (its brute-force flock-ref oracle, restated in C)
    on all host cores. A full step at 1M birds takes ~24 s of CPU, so each
    step here is a bounded sample of one: the brute-force decide of a random
    subset of that step's deciding birds, plus integrate of every bird. The
    line reports what ran: `ms_per_step` is the measured wall time of one
    sampled step, and `value` is the rate of the work it did, in bird-update
    equivalents per second (the sample's fraction of a full step's work x n,
    over its wall time), which equals n over the extrapolated full-step time
    (`extrapolated_step_s`)."""
    if rank != 0:
        return
    from oracle import pyoracle as o

    words = o.scatter(args.birds, args.seed)
    per_step = max(0.05, 90.0 / max(1, args.steps + args.warmup))
    for _ in range(args.warmup):
        cpu_sample(words, 0.02)
    walls, steps_s, fracs = [], [], []
    for s in range(args.steps):
        r = cpu_sample(words, per_step, seed=s)
        walls.append(r["sample_wall_s"])
        steps_s.append(r["extrapolated_step_s"])
        fracs.append(r["sample_wall_s"] / r["extrapolated_step_s"])
    ext = statistics.mean(steps_s)
    value = args.birds / ext
    world = int(os.environ.get("WORLD_SIZE", "1"))
    out = {"metric": METRIC, "impl": "reference", "value": value, "unit": "bird-updates/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(walls) * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (flock-ref gen scatter: SplitMix64, density 0.5)",
           "config": workload_config(args.birds, args.seed, world),
           "extrapolated_step_s": ext, "work_fraction_per_step": statistics.mean(fracs),
           "how": "each timed step is a bounded sample of one full step (the brute-force decide of a random subset "
                  "of its deciding birds, each against all birds, plus integrate of every bird); ms_per_step is "
                  "that sample's measured wall time; value = the sample's share of a full step's work x birds / "
                  "its wall time = birds / extrapolated_step_s",
           "cpu_baseline": {"value": value, "unit": "bird-updates/s", "cores": r["cores"], "kind": "port",
                            "sample": f"per step: {r['sample']}; {args.steps} sampled steps"},
           "e2e": {"value": value, "unit": "bird-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def ref_gpu(n: int, seed: int, steps: int, warmup: int, device: int, words=None) -> dict:
    """Reported baseline, not our product: the reference's own CUDA kernels
    (cuda/flock.cu compiled unchanged for sm_103a, oracle/_ref) on this GPU,
    driven with the reference's host loop and per-pass timing protocol
    (cuda/flock.cu:447-492), on the same starting state."""
    try:
        from oracle import ref_kernels as rk

        drv = rk.Driver(device)
        try:
            t = rk.time_reference(drv, n, seed, steps, warmup, words=words)
        finally:
            drv.close()
    except Exception as e:  # the cubin is built only where the reference is mounted
        return {"unavailable": f"{type(e).__name__}: {e}"}
    return {"kind": "reference kernels (cuda/flock.cu for sm_103a, same GPU)", "birds": n, "seed": seed,
            "steps": steps, "warmup": warmup, "value": t["bird_steps_per_s"], "unit": "bird-updates/s",
            "ms_per_step": t["step_total"],
            "passes_ms": {k: round(t[k], 5) for k in ("grid_histogram", "grid_scan", "grid_scatter", "decide",
                                                      "integrate")},
            "how": "memset + 7 launches per step on one stream, CUDA events between passes, mean GPU ms per pass "
                   "over the timed steps (the reference's own protocol; no L2 flush)"}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def bench_plain(m, args, dist, local):
    n, K, W = args.birds, args.steps, max(3, args.warmup)
    words = m.generate(n, args.seed)
    f = m.Flock(words, 0.0, device=local)
    if args.decide == "staged":
        f.tune_decide(1)
    f.step(W)
    barrier(dist)
    with ClockSampler(local) as clk:
        ms = f.time_steps(K, FLUSH_BYTES)
    barrier(dist)
    total_ms = float(ms.sum())
    due0, cand0, pairs0 = f.counters()
    # per-pass shares from an eager run with events between passes (same state continues)
    passes = f.step_timed(10, 0)
    due1, cand1, pairs1 = f.counters()
    # the next step's f32 error against the same step evaluated in FP64 (flk_step_f64)
    _, fp64 = f.step_f64()
    f.close()
    return dict(ms=ms, total_ms=total_ms, clocks=clk.summary(), passes=passes, fp64=fp64,
                due_frac=(due1 - due0) / (10 * n), cand_per_due=(cand1 - cand0) / max(1, due1 - due0),
                pairs_per_due=(pairs1 - pairs0) / max(1, due1 - due0), due_total=due0)


def decide_rates(r, n):
    """decide's work rates over the eager passes' decide time: candidate tests/s
    and true pairs (within 2R) per second, with the per-bird figures."""
    due_per_step = r["due_frac"] * n
    dec_s = r["passes"]["decide_ms"] / 1e3
    return {"candidates_per_deciding_bird": r["cand_per_due"], "pairs_in_2R_per_deciding_bird": r["pairs_per_due"],
            "deciding_per_step": due_per_step,
            "candidate_tests_per_s": r["cand_per_due"] * due_per_step / dec_s if dec_s > 0 else None,
            "pairs_per_s": r["pairs_per_due"] * due_per_step / dec_s if dec_s > 0 else None}


def pass_bandwidths(r, n):
    """Algorithmic bytes of each streaming pass / its eager time (GB/s): hash reads
    a position and writes key + rank (24 B/bird); scatter + sort read key, rank,
    bird index, sort key and the state and write the state, heading and the
    deciding birds' records (8+4+4+8+68 + 8+68+16 + 48 f B/bird); integrate
    reads position, velocity, steering and writes position, velocity (80 B/bird)."""
    p, f = r["passes"], r["due_frac"]
    def gbs(bytes_per_bird, ms):
        return round(bytes_per_bird * n / (ms / 1e3) / 1e9, 1) if ms > 0 else None
    return {"hash": gbs(24, p["hash_ms"]), "scatter_sort": gbs(184 + 48 * f, p["sort_ms"]),
            "integrate": gbs(80, p["integrate_ms"])}


# decide's warp instructions per launch at 1M birds (seed 1), from the committed
# ncu summary (smsp__inst_executed.sum) of the decide kernel as of commit
# PROFILED_AT; 4 warp instructions per clock per SM peak. Both this figure and
# the step traffic in profiles/traffic_step_1m.txt are re-taken whenever the
# kernels change.
DECIDE_INST_1M = 109.0e6
PROFILED_AT = "2758cb7"
GB300_SMS = 152


def dominant_kernel(r, n, seed):
    """decide's share of the step (live) and its limiter: instruction issue. For
    the 1M-bird, seed-1 step, the achieved issue rate is the profiled
    instruction count over the live decide time, against 4 warp instructions
    per clock per SM at the sampled SM clock."""
    p = r["passes"]
    out = {"name": "k_decide", "share_of_step": p["decide_ms"] / p["total_ms"] if p["total_ms"] > 0 else None,
           "bound": "instruction issue (not HBM: ~65 MB of DRAM traffic per launch)",
           "evidence": "profiles/decide_1m_current.txt"}
    mhz = (r["clocks"] or {}).get("sm_mhz")
    if (n, seed) == (1_000_000, 1) and p["decide_ms"] > 0 and mhz:
        achieved = DECIDE_INST_1M / (p["decide_ms"] / 1e3)
        peak = 4.0 * GB300_SMS * mhz * 1e6
        out.update({"issue_achieved": achieved, "issue_peak": peak, "issue_unit": "warp instructions/s",
                    "issue_frac": achieved / peak,
                    "instructions_source": f"{DECIDE_INST_1M:.4g} warp instructions per launch from "
                                           f"profiles/decide_1m_current.txt (profiled at commit {PROFILED_AT}) "
                                           f"over this run's decide time"})
    return out


def bench_configs(m, local) -> list:
    """The plain step at the other two single-flock sizes, each with its own
    steps protocol: 100,000 birds (seed 1, 20 warm-up + 20 timed) and
    16,777,216 birds (seed 7, 10 + 50). Timed as the headline (one graph
    launch per step after an L2 flush, CUDA events), beside the reference's
    kernels on the same GPU and the same starting state."""
    rows = []
    for n, seed, warm, steps in [(100_000, 1, 20, 20), (16_777_216, 7, 10, 50)]:
        words = m.generate(n, seed)
        f = m.Flock(words, 0.0, device=local)
        f.step(warm)
        with ClockSampler(local) as clk:
            ms = f.time_steps(steps, FLUSH_BYTES)
        f.close()
        v = n * steps / (float(ms.sum()) / 1e3)
        ref = ref_gpu(n, seed, warm + steps, warm, local, words=words)
        row = {"workload": f"plain single-flock step, {n:,} birds, seed {seed}", "birds": n, "seed": seed,
               "warmup": warm, "steps": steps, "value": v, "unit": "bird-updates/s",
               "ms_per_step": float(ms.mean()), "step_ms_p50": float(np.median(ms)), "clocks": clk.summary(),
               "ref_gpu": ref}
        if "value" in ref:
            row["speedup_vs_ref_gpu"] = v / ref["value"]
        rows.append(row)
        del words
    return rows


def bench_multi_step(m, args, local):
    """The same workload as the library runs it for flk_step(K): 10-step CUDA
    graphs, each step's integrate also counting the next step's grid, no L2
    flush between steps (device time, CUDA events). Not the headline: the
    headline flushes L2 before every single-step launch."""
    n, K = args.birds, args.steps
    b = m.Batch(device=local)
    b.add(m.generate(n, args.seed))
    b.step(max(10, args.warmup))  # warm-up and graph capture
    ms = b.time_steps(K)
    b.close()
    return {"value": n * K / (ms / 1e3), "unit": "bird-updates/s", "ms_per_step": ms / K,
            "how": f"{K} steps in 10-step CUDA graphs (fused integrate and next hash), no L2 flush between steps"}


def bench_e2e(m, args, local):
    """Through the C ABI with host buffers: upload, K steps, download."""
    n, K = args.birds, args.steps
    words = m.generate(n, args.seed)
    out = np.empty_like(words)
    with m.pinned(words, out):
        # one untimed pass first so lazy CUDA initialisation is not timed
        g = m.Flock(words[:1024].copy(), 0.0, device=local)
        g.step(1)
        g.close()
        runs = []
        for _ in range(3):  # the median of three whole runs (host wall clock)
            t0 = time.perf_counter()
            f = m.Flock(words, 0.0, device=local)
            f.step(K)
            f.read(out)
            t1 = time.perf_counter()
            f.close()
            runs.append(t1 - t0)
    s = float(np.median(runs))
    return {"value": n * K / s, "unit": "bird-updates/s", "h2d_bytes_per_step": n * WORDS * 4 / K,
            "d2h_bytes_per_step": n * WORDS * 4 / K,
            "runs_ms": [round(x * 1e3, 2) for x in runs],
            "how": f"flk_open_host (H2D of {n * 60 / 1e6:.0f} MB, pinned) + flk_step({K}) + flk_read_host "
                   f"(D2H) through the C ABI, host wall clock, median of 3 runs {s * 1e3:.1f} ms"}


def bench_batched(m, args, local):
    rng = np.random.default_rng(3)
    sizes = log_uniform_sizes(rng, 256, 1_000, 200_000)
    K = args.batched_steps
    flocks = [m.generate(int(nf), 3 + k) for k, nf in enumerate(sizes)]
    total = int(sizes.sum())
    from murmuration_kernels_gb300 import autotune

    # launch shapes for this mix, tuned on a copy: the tuner's trials advance
    # the flocks, and the timed batch must start from the same states as the
    # one-at-a-time runs below
    t = m.Batch(device=local)
    for w in flocks:
        t.add(w)
    tuned = autotune.tune(t, steps=10, use_cache=False)
    t.close()
    b = m.Batch(device=local)
    for w in flocks:
        b.add(w)
    b.tune(**{k: v for k, v in tuned["shape"].items()})
    b.step(10)  # warm-up (graph capture), as the one-at-a-time runs
    ms_batched = b.time_steps(K)
    passes = b.step_timed(5, 0)
    b.close()
    # the same flocks one at a time through the plain step (same graphs, one flock each)
    ms_plain = 0.0
    for w in flocks:
        p = m.Batch(device=local)
        p.add(w)
        p.step(10)
        ms_plain += p.time_steps(K)
        p.close()
    v_b = total * K / (ms_batched / 1e3)
    v_p = total * K / (ms_plain / 1e3)
    return {"value": v_b, "unit": "bird-updates/s", "flocks": 256, "birds": total, "steps": K,
            "ms_per_step": ms_batched / K, "plain_one_at_a_time": v_p, "speedup_vs_plain": v_b / v_p,
            "passes_ms": {k: round(v, 5) for k, v in passes.items() if k.endswith("_ms")},
            "autotuned": {"shape": tuned["shape"], "trials": tuned["trials"]},
            "config": "256 flocks, n log-uniform [1e3, 2e5] (seed 3), flock k seed 3+k, 10-step CUDA graphs"}


def bench_served(m, args, local):
    rng = np.random.default_rng(5)
    R = args.requests
    sizes = log_uniform_sizes(rng, R, 2_000, 1_000_000)
    steps = rng.integers(10, 501, size=R)
    gaps = rng.exponential(1.0 / args.rate, size=R)
    arrivals = np.cumsum(gaps) - gaps[0]
    states = [m.generate(int(nf), 5 + k) for k, nf in enumerate(sizes)]
    outs = [np.empty_like(w) for w in states]
    demand = float(np.sum(sizes * steps))
    budget = 150 << 30
    lat = [0.0] * R
    with m.pinned(*states, *outs):
        with m.Pool(budget, chunk_steps=args.chunk, device=local) as pool:
            # warm the pool (graph capture, CUDA init) with a tiny request
            pool.wait(pool.submit(m.generate(1000, 99), 12))
            tickets = [None] * R
            t0 = time.perf_counter()

            def feeder():
                for k in range(R):
                    dt = t0 + arrivals[k] - time.perf_counter()
                    if dt > 0:
                        time.sleep(dt)
                    tickets[k] = pool.submit(states[k], int(steps[k]), out=outs[k])

            th = threading.Thread(target=feeder)
            th.start()
            th.join()
            for k in range(R):
                _, _, lat[k] = pool.wait(tickets[k])
            t_end = time.perf_counter()
            # the same requests all at once: the pool's capacity under full load
            t1 = time.perf_counter()
            tk = [pool.submit(states[k], int(steps[k]), out=outs[k]) for k in range(R)]
            lat_sat = [pool.wait(t)[2] for t in tk]
            span_sat = time.perf_counter() - t1
        span = t_end - t0
    # the same requests one at a time through the plain step, FCFS on the same arrivals
    service = []
    for k in range(R):
        s0 = time.perf_counter()
        f = m.Flock(states[k], 0.0, device=local)
        f.step(int(steps[k]))
        f.read(outs[k])
        f.close()
        service.append(time.perf_counter() - s0)
    finish, lat_seq = 0.0, []
    for k in range(R):
        start = max(arrivals[k], finish)
        finish = start + service[k]
        lat_seq.append((finish - arrivals[k]) * 1e3)
    span_seq = finish - arrivals[0]
    p = lambda xs, q: float(np.percentile(np.asarray(xs), q))
    return {"value": demand / span, "unit": "bird-updates/s", "requests": R, "rate_per_s": args.rate,
            "p50_ms": p(lat, 50), "p99_ms": p(lat, 99),
            "sequential_plain": {"value": demand / span_seq, "p50_ms": p(lat_seq, 50), "p99_ms": p(lat_seq, 99)},
            "speedup_vs_plain": (demand / span) / (demand / span_seq),
            "saturated": {"value": demand / span_sat, "p50_ms": p(lat_sat, 50), "p99_ms": p(lat_sat, 99),
                          "sequential_plain": demand / sum(service),
                          "speedup_vs_plain": sum(service) / span_sat,
                          "how": "the same requests submitted together; the plain arm runs them back to back"},
            "config": f"Poisson arrivals {args.rate}/s (seed 5), n log-uniform [2e3, 1e6], steps U[10, 500], "
                      f"150 GB admission budget, {args.chunk}-step fold-in chunks"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--birds", type=int, default=1_000_000)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the batched / served / CPU / reference-kernel / other-size measurements")
    ap.add_argument("--batched-steps", type=int, default=30)
    ap.add_argument("--requests", type=int, default=64)
    ap.add_argument("--rate", type=float, default=100.0)
    ap.add_argument("--chunk", type=int, default=10)
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--decide", choices=["direct", "staged"], default="direct",
                    help="the headline step's decide kernel (staged: neighbourhoods in shared memory)")
    args = ap.parse_args()

    dist, rank, world, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, dist, rank)
        return

    import murmuration_kernels_gb300 as m

    r = bench_plain(m, args, dist, local)
    n, K = args.birds, args.steps
    ms_max, units = aggregate(dist, r["total_ms"], float(n * K))
    value = units / (ms_max / 1e3)
    ms_per_step = ms_max / K
    f = r["due_frac"]
    b_alg = 60 + 32 + 28 * f + 16
    peak, peak_kind = peak_hbm()
    achieved = b_alg * n / (ms_per_step / 1e3) / 1e9
    # the committed ncu figure is for the 1M-bird, seed-1 step only
    traffic = step_traffic_bytes() if (n, args.seed) == (1_000_000, 1) else None
    out = {
        "metric": METRIC, "value": value, "unit": "bird-updates/s", "n_gpus": world, "steps": K,
        "warmup": max(3, args.warmup), "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (flock-ref gen scatter: SplitMix64, density 0.5)",
        "config": workload_config(n, args.seed, world),
        "roofline": {"bound": "hbm", "kernel": "whole step (5 launches in one graph launch)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "bytes_per_update": b_alg, "due_fraction": f,
                     "traffic": traffic,
                     "traffic_source": f"{os.path.relpath(TRAFFIC, ROOT)} (ncu capture of one timed step; "
                                       f"profiled at commit {PROFILED_AT})" if traffic else None},
        # what bounds the step: decide's share of the eager pass times (live) and its
        # limiter, from the committed ncu summary of the same workload
        "dominant_kernel": dominant_kernel(r, n, args.seed),
        "passes_ms": {k: round(v, 5) for k, v in r["passes"].items() if k.endswith("_ms")},
        "decide": decide_rates(r, n),
        "passes_gbs": pass_bandwidths(r, n),
        # a timed step has no hash pass of its own (the previous integrate counted its grid)
        "gpu_launches": (m.kernels_per_step() - 1) * K,
        "gpu_launches_how": "kernels in the timed steps' graph launches: place, scatter, sort, decide and "
                            "integrate per step (the L2-flush kernel between steps not counted)",
        "fp64_error": dict(r["fp64"], how="one more f32 step against the same step in FP64 from the same state "
                                          "(max relative position / velocity error over all birds; neighbour-count "
                                          "mismatches)"),
        "clocks": r["clocks"],
        "step_ms_p50": float(np.median(r["ms"])), "step_ms_min": float(r["ms"].min()),
    }
    if rank == 0:
        out["e2e"] = bench_e2e(m, args, local)
        out["multi_step"] = bench_multi_step(m, args, local)
        if not args.no_extra:
            # the reference's own kernels on this GPU at the headline workload, with
            # the reference's protocol for it (20 warm-up + 100 timed steps)
            out["ref_gpu"] = ref_gpu(n, args.seed, 120, 20, local, words=m.generate(n, args.seed))
            if "value" in out["ref_gpu"]:
                out["ref_gpu"]["speedup"] = value / out["ref_gpu"]["value"]
            out["configs"] = bench_configs(m, local)
        if not args.no_extra:
            out["batched"] = bench_batched(m, args, local)
            out["served"] = bench_served(m, args, local)
            out["cpu_baseline"] = cpu_sample(m.generate(n, args.seed), args.cpu_budget)
            out["cpu_grid"] = cpu_grid_steps(m.generate(n, args.seed), 2 if n <= 4_000_000 else 1)
        print(json.dumps(out), flush=True)
    barrier(dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
