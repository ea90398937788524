#!/usr/bin/env python3
"""Generates golden fixtures from the REFERENCE's own CUDA kernels.

The reference's cuda/flock.cu is compiled unchanged for sm_103a into
oracle/_ref/flock_ref_sm103a.cubin (oracle/Makefile, target `ref`, run where the
reference project is mounted); oracle/ref_kernels.py drives its kernels exactly
as the reference's host loop does, on the reference generator's starting
states. This script writes:

  ref_cuda_2000_s1.npz     2000 birds, seed 1 (scripts/parity.sh's case):
                           input, state after 1 and after 100 steps, and the
                           first step's bucket keys and offsets
  ref_cuda_100k_s1.npz     100,000 birds, seed 1, one step: SHA-256 digests of
                           the bucket keys, offsets and neighbour counts, plus
                           every 97th bird's full state

Run on a machine with a GPU (the fixtures are committed; tests only read them):
    python tests/golden/make_reference_fixtures.py OUTDIR
    python tests/golden/make_reference_fixtures.py --time N SEED STEPS WARMUP
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.ref_kernels import Driver, run_reference, time_reference  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main(outdir: str):
    from oracle import pyoracle as o

    os.makedirs(outdir, exist_ok=True)
    drv = Driver()
    w = o.scatter(2000, 1)
    t1, out1, keys1, offs1 = run_reference(drv, w, 0.0, 1)
    t100, out100, _, _ = run_reference(drv, w, 0.0, 100)
    np.savez_compressed(os.path.join(outdir, "ref_cuda_2000_s1.npz"), input=w, time1=np.float32(t1), out1=out1,
                        keys1=keys1, offsets1=offs1, time100=np.float32(t100), out100=out100)
    w = o.scatter(100_000, 1)
    t, out, keys, offs = run_reference(drv, w, 0.0, 1)
    pick = np.arange(0, 100_000, 97)
    np.savez_compressed(os.path.join(outdir, "ref_cuda_100k_s1.npz"), time1=np.float32(t), pick=pick,
                        out1_pick=out[pick], keys_sha=sha(keys), offsets_sha=sha(offs),
                        neighbours_sha=sha(out[:, 13].view(np.uint32)),
                        next_decision_sha=sha(out[:, 12]))
    print("wrote fixtures to", outdir)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--time":
        # python tests/golden/make_reference_fixtures.py --time N SEED STEPS WARMUP
        import json

        n, seed, steps, warmup = (int(x) for x in sys.argv[2:6])
        print(json.dumps({"birds": n, "seed": seed, "steps": steps, "warmup": warmup,
                          **time_reference(Driver(), n, seed, steps, warmup)}))
    else:
        main(sys.argv[1] if len(sys.argv) > 1 else HERE)
