"""Multi-GPU is replicas only: bench.py under torchrun runs one independent
flock per rank, with a barrier, max time over ranks and summed bird-updates.
The rank bookkeeping is tested here with the gloo backend, world size 2, on CPU.
"""
from __future__ import annotations

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    dist, r, w, local = bench.dist_setup()
    try:
        # rank r "took" (r + 1) * 10 ms for 1e6 bird-updates
        ms, units = bench.aggregate(dist, (r + 1) * 10.0, 1e6)
        bench.barrier(dist)
        q.put((r, w, local, ms, units, dist.get_backend()))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_over_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    for r, w, local, ms, units, backend in out:
        assert w == 2 and local == r and backend == "gloo"
        assert ms == 20.0          # max over ranks
        assert units == 2e6        # sum over ranks
    # whole-job throughput as bench.py reports it
    assert out[0][4] / (out[0][3] / 1e3) == pytest.approx(1e8)


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    saved = {k: os.environ.pop(k, None) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    try:
        dist, rank, world, local = bench.dist_setup()
        assert dist is None and (rank, world, local) == (0, 1, 0)
        assert bench.aggregate(None, 5.0, 7.0) == (5.0, 7.0)
    finally:
        for k, v in saved.items():
            if v is not None:
                os.environ[k] = v


def test_reference_arm_prints_the_contract_line():
    """bench.py --impl reference (the oracle port timed on the host cores) runs
    without a GPU and prints one JSON line with the reference-arm fields."""
    import json
    import subprocess

    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--birds", "20000",
                        "--steps", "2", "--warmup", "1", "--cpu-budget", "0.5"],
                       capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "bird-updates/s" and d["value"] > 0
    assert d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["birds"] == 20000


def test_clock_summary_parses_nvidia_smi_rows(tmp_path):
    """bench.py's clock record: median SM clock under load, the maximum, and every
    throttle reason seen active during the region."""
    sys.path.insert(0, ROOT)
    import bench

    rows = ["0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
            "0, 1995, 2070, 1200.5, 0x4, Not Active, Not Active, Not Active, Active",
            "0, 2040, 2070, 1100.0, 0x0, Not Active, Not Active, Not Active, Not Active",
            "garbage line"]
    path = tmp_path / "clocks.csv"
    path.write_text("\n".join(rows) + "\n")
    c = bench.ClockSampler(0)
    c.proc, c.path = object(), str(path)
    s = c.summary()
    assert s == {"sm_mhz": 2040.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    assert not path.exists()


def test_step_traffic_comes_from_the_committed_profile():
    """roofline.traffic is the committed ncu figure for the 1M-bird step: the
    summary's step_dram_bytes line, equal to its per-kernel table's sum."""
    sys.path.insert(0, ROOT)
    import bench

    t = bench.step_traffic_bytes()
    assert t is not None and t > 0
    total = 0.0
    for line in open(bench.TRAFFIC):
        parts = line.split()
        if not parts or not parts[0].startswith("k_") or len(parts) < 4:
            continue
        try:  # table rows: kernel, time, DRAM read MB, DRAM write MB, ...
            total += (float(parts[2]) + float(parts[3])) * 1e6
        except ValueError:
            continue
    assert abs(total - t) / t < 1e-3
