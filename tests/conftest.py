"""Shared fixtures. GPU tests are marked `gpu`; everything else runs on CPU.

The native library and the oracle are built in-tree on first use when their
outputs are missing or older than their sources.
"""
from __future__ import annotations

import glob
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


@pytest.fixture(scope="session")
def native():
    import murmuration_kernels_gb300 as m
    from murmuration_kernels_gb300 import build as b

    srcs = glob.glob(os.path.join(b.CSRC, "*")) + [m.HEADER]
    if _stale(m.LIB_PATH, srcs) or _stale(m.CLI_PATH, srcs):
        b.build()
    m.lib()
    return m


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle as o

    srcs = glob.glob(os.path.join(o.HERE, "*.c")) + glob.glob(os.path.join(o.HERE, "*.h"))
    if _stale(o.LIB, srcs) or _stale(o.CLI, srcs):
        o.build()
    o.lib()
    return o
