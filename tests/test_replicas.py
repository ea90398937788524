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
