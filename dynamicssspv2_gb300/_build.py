"""In-tree build of the dsssp library, its command line, and the CPU oracle.

Outputs (git-ignored):
    dynamicssspv2_gb300/_lib/libdsssp.so   C ABI of include/dsssp.h (CUDA for sm_103a + host code)
    dynamicssspv2_gb300/_lib/dsssp_main    drop-in command line for SSSPmainForUndirected.cu
    oracle/liboracle.so                    CPU oracle (test infrastructure)
    oracle/_ref/*                          the reference compiled from its own sources (only
                                           where those sources are present)

Translation units compile in parallel; a target is rebuilt only when a source is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = ROOT / "_build"
LIB = PKG / "_lib"
INCLUDE = ROOT / "include"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function"]

CUDA_UNITS = ["update.cu", "graph.cu", "noalloc.cu"]
HOST_UNITS = ["gen.cpp", "textio.cpp", "binio.cpp", "serve.cpp", "autotune.cpp"]
HEADERS = ["engine.cuh", "host_common.h"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the dsssp library needs the CUDA toolkit")


def _newer(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def _run_parallel(jobs: list[list[str]]) -> None:
    procs = [(cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for cmd in jobs]
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, out))
    if failed:
        msg = "\n".join(f"$ {' '.join(c)}\n{o}" for c, o in failed)
        raise RuntimeError(f"build failed:\n{msg}")


def build_library(verbose: bool = False) -> Path:
    """Compiles libdsssp.so and dsssp_main; returns the library path."""
    BUILD.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = [CSRC / h for h in HEADERS] + [INCLUDE / "dsssp.h"]
    jobs, objs = [], []
    for unit in CUDA_UNITS:
        src, obj = CSRC / unit, BUILD / (Path(unit).stem + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)])
    for unit in HOST_UNITS:
        src, obj = CSRC / unit, BUILD / (Path(unit).stem + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", str(src), "-o", str(obj)])
    if verbose:
        for j in jobs:
            print(" ".join(j), file=sys.stderr)
    _run_parallel(jobs)
    lib = LIB / "libdsssp.so"
    if _newer(lib, objs):
        _run_parallel([[nvcc] + ARCH + ["-shared", "-o", str(lib)] + [str(o) for o in objs] + ["-lgomp"]])
    cli = LIB / "dsssp_main"
    if _newer(cli, [CSRC / "dsssp_main.cpp", lib, INCLUDE / "dsssp.h"]):
        _run_parallel([["g++", "-O2", "-std=c++17", "-o", str(cli), str(CSRC / "dsssp_main.cpp"), f"-L{LIB}",
                        "-ldsssp", "-Wl,-rpath,$ORIGIN"]])
    return lib


def build_oracle() -> None:
    """Compiles the CPU oracle; also the reference's own code where its sources exist (the
    oracle's Makefile knows where they lie; DSSSP_REFERENCE overrides it)."""
    subprocess.run(["make", "-s", "-C", str(ORACLE), "all", "ref-if-present"], check=True)


def build_all(verbose: bool = False) -> None:
    build_library(verbose)
    build_oracle()


if __name__ == "__main__":
    build_all(verbose=True)
