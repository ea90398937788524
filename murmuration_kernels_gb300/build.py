"""Builds the native parts in-tree: the sm_103a kernels + C-ABI library, the CLI.

    python -m murmuration_kernels_gb300.build        (or __graft_entry__.build())

Outputs go to murmuration_kernels_gb300/_build/ (git-ignored):
    libflock_gb300.so   kernels (flock_engine.cu) + C ABI (flock_abi.cpp)
    flock_gb300         the drop-in CLI

Translation units compile in parallel; one -gencode (sm_103a). Host code is
built with -ffp-contract=off so no compiler contracts f32 arithmetic into
FMAs on either host architecture.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
REPO = os.path.dirname(HERE)
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home() -> str:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env and os.path.isdir(env):
        return env
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def commands(verbose_ptxas: bool = False) -> tuple[list[list[str]], list[list[str]]]:
    ch = cuda_home()
    nvcc = os.path.join(ch, "bin", "nvcc")
    inc = os.path.join(ch, "include")
    os.makedirs(OUT, exist_ok=True)
    eng_o = os.path.join(OUT, "flock_engine.o")
    noalloc_o = os.path.join(OUT, "flock_noalloc.o")
    abi_o = os.path.join(OUT, "flock_abi.o")
    lib = os.path.join(OUT, "libflock_gb300.so")
    cli = os.path.join(OUT, "flock_gb300")
    cu = [nvcc, ARCH, "-lineinfo", "-O3", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-c", os.path.join(CSRC, "flock_engine.cu"), "-o", eng_o]
    if verbose_ptxas:
        cu.insert(1, "-Xptxas=-v")
    # extra nvcc flags, e.g. FLK_NVCC_FLAGS=-Xptxas=-v for register and spill reports
    extra = os.environ.get("FLK_NVCC_FLAGS", "").split()
    cu[1:1] = extra
    cu_na = cu[:cu.index("-c")] + ["-c", os.path.join(CSRC, "flock_noalloc.cu"), "-o", noalloc_o]
    cxx = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I" + inc,
           "-c", os.path.join(CSRC, "flock_abi.cpp"), "-o", abi_o]
    link = [nvcc, ARCH, "-shared", "-o", lib, eng_o, noalloc_o, abi_o, "-Xcompiler", "-fPIC", "-lpthread"]
    cli_cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + inc, os.path.join(CSRC, "flock_cli.cpp"),
               "-o", cli, "-L" + OUT, "-lflock_gb300", "-L" + os.path.join(ch, "lib64"), "-lcudart",
               "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + os.path.join(ch, "lib64")]
    return [cu, cu_na, cxx], [link, cli_cmd]


def build(verbose_ptxas: bool = False) -> str:
    """Compiles the library and CLI; returns the library path."""
    parallel, serial = commands(verbose_ptxas)
    with ThreadPoolExecutor(max_workers=len(parallel)) as ex:
        list(ex.map(_run, parallel))
    for cmd in serial:
        _run(cmd)
    return os.path.join(OUT, "libflock_gb300.so")


if __name__ == "__main__":
    print(build("-v" in sys.argv))
