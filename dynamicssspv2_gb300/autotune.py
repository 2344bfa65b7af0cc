"""Autotuner of the update's launch and frontier-switch settings (binding of the native one).

The search runs in C++ behind the C ABI (`dsssp_autotune`, csrc/autotune.cpp): for a graph
and a representative change batch it times each candidate setting -- edges per thread item
and CTA-chunk thresholds (the degree buckets), subtree-walk depth before pointer jumping, CTA
size and residency, solo-step width, near-far bucket widths scaled by the batch's mean
weight -- on the same batch from the same starting state (device snapshot and restore), sets
the fastest on the graph and caches it per size class (log2 vertices, log2 adjacency entries,
log2 batch size) in a text file.  The command line (--autotune) and the server (tune_cache)
read the same cache.  The reference has no tunables (THREADS_PER_BLOCK is a compile-time
macro, SSSPmainForUndirected.cu:11).

Tuning takes a device snapshot of the graph (replacing any snapshot taken before) and leaves
the graph restored to its state before tuning.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import CHANGE_DTYPE, Graph, Opts, _check, _lib, abi_sizes

TUNED_FIELDS = ("small_deg", "large_deg", "chunk", "bfs_levels", "block", "ctas_per_sm", "delta", "solo_waves",
                "group_ctas", "group_waves", "warp_agg", "auto_rounds")


class TuneResult(C.Structure):
    _fields_ = [("key", C.c_char * 32), ("opts", Opts), ("ms", C.c_double), ("trials", C.c_int32),
                ("cached", C.c_int32)]


if abi_sizes()[4] != C.sizeof(TuneResult):
    raise ImportError(f"the library's dsssp_tune_result is {abi_sizes()[4]} bytes, this binding's {C.sizeof(TuneResult)}")

_lib.dsssp_autotune.restype = C.c_int
_lib.dsssp_autotune.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_char_p, C.c_int32, C.c_int32,
                                C.POINTER(TuneResult)]
_lib.dsssp_autotune_lookup.restype = C.c_int
_lib.dsssp_autotune_lookup.argtypes = [C.c_void_p, C.c_int64, C.c_char_p, C.POINTER(TuneResult)]
_lib.dsssp_tune_size_class.restype = C.c_int
_lib.dsssp_tune_size_class.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_char_p, C.c_size_t]
_lib.dsssp_tune_candidates.restype = C.c_int
_lib.dsssp_tune_candidates.argtypes = [C.POINTER(Opts), C.c_void_p, C.c_int64, C.POINTER(Opts), C.c_int32,
                                       C.POINTER(C.c_int32)]


def default_cache_path() -> Path:
    env = os.environ.get("DSSSP_AUTOTUNE_CACHE")
    if env:
        return Path(env)
    return Path(os.path.expanduser("~")) / ".cache" / "dsssp" / "autotune.txt"


def size_class(n: int, entries: int, k: int) -> str:
    buf = C.create_string_buffer(32)
    _check(_lib.dsssp_tune_size_class(int(n), int(entries), int(k), buf, 32), "tune_size_class")
    return buf.value.decode()


def candidates(base: Opts, changes: np.ndarray) -> list[Opts]:
    """The settings the tuner times for this batch, starting from base."""
    ch = np.ascontiguousarray(changes, CHANGE_DTYPE)
    out = (Opts * 64)()
    cnt = C.c_int32()
    _check(_lib.dsssp_tune_candidates(C.byref(base), ch.ctypes.data if len(ch) else None, len(ch), out, 64,
                                      C.byref(cnt)), "tune_candidates")
    return list(out[: cnt.value])


def _opts_dict(o: Opts) -> dict:
    return {f: int(getattr(o, f)) for f in TUNED_FIELDS}


class Autotuner:
    def __init__(self, cache_path: str | os.PathLike | None = None, reps: int = 3):
        self.path = Path(cache_path) if cache_path else default_cache_path()
        self.reps = reps

    def tune(self, graph: Graph, changes: np.ndarray, force: bool = False) -> dict:
        """Sets the fastest setting for (graph, changes) on the graph and returns {"key", "opts",
        "ms", "trials", "cached"}; a cached size class is applied without timing."""
        self.path.parent.mkdir(parents=True, exist_ok=True)
        ch = np.ascontiguousarray(changes, CHANGE_DTYPE)
        r = TuneResult()
        _check(_lib.dsssp_autotune(graph.handle, ch.ctypes.data, len(ch), str(self.path).encode(), int(self.reps),
                                   1 if force else 0, C.byref(r)), "autotune")
        return {"key": r.key.decode(), "opts": _opts_dict(r.opts), "ms": r.ms, "trials": int(r.trials),
                "cached": bool(r.cached)}
