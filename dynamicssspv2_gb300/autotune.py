"""Autotuner for the update kernels' launch tunables.

For a graph and a representative change batch it times a short list of candidate settings
(edges per thread item, CTA-chunk thresholds, subtree-walk depth before pointer jumping, CTA
size and residency, near-far bucket width), each on the same batch from the same starting
state (device snapshot and restore), keeps the fastest, and caches it per size class --
(log2 vertices, log2 adjacency entries, log2 batch size) -- in a JSON file, so later graphs
of the same class skip the search.  The reference has no tunables (THREADS_PER_BLOCK is a compile-time macro,
SSSPmainForUndirected.cu:11).

Tuning takes a device snapshot of the graph (replacing any snapshot taken before) and leaves
the graph restored to its state before tuning.
"""
from __future__ import annotations

import json
import math
import os
from pathlib import Path

import numpy as np

from . import Graph, Opts

CANDIDATES = [
    {},
    {"small_deg": 8},
    {"small_deg": 4, "large_deg": 1024, "chunk": 1024},
    {"small_deg": 4, "large_deg": 4096, "chunk": 2048},
    {"bfs_levels": 0},
    {"bfs_levels": 8},
    {"block": 128},
    {"ctas_per_sm": 2},
]

TUNED_FIELDS = ("small_deg", "large_deg", "chunk", "bfs_levels", "block", "ctas_per_sm", "delta")


def default_cache_path() -> Path:
    env = os.environ.get("DSSSP_AUTOTUNE_CACHE")
    if env:
        return Path(env)
    return Path(os.path.expanduser("~")) / ".cache" / "dsssp" / "autotune.json"


def size_class(n: int, entries: int, k: int) -> str:
    lg = lambda x: int(round(math.log2(max(int(x), 1))))  # noqa: E731
    return f"v{lg(n)}_e{lg(entries)}_b{lg(k)}"


class Autotuner:
    def __init__(self, cache_path: str | os.PathLike | None = None, candidates=None, reps: int = 2):
        self.path = Path(cache_path) if cache_path else default_cache_path()
        self.candidates = candidates if candidates is not None else CANDIDATES
        self.reps = reps
        try:
            self.cache = json.loads(self.path.read_text())
        except (OSError, ValueError):
            self.cache = {}

    def save(self) -> None:
        self.path.parent.mkdir(parents=True, exist_ok=True)
        tmp = self.path.with_suffix(".tmp")
        tmp.write_text(json.dumps(self.cache, indent=1, sort_keys=True))
        tmp.replace(self.path)

    @staticmethod
    def _apply(base: Opts, overrides: dict) -> Opts:
        o = Opts()
        for name, _ in Opts._fields_:
            setattr(o, name, getattr(base, name))
        for k, v in overrides.items():
            setattr(o, k, v)
        return o

    @staticmethod
    def near_far_candidates(changes: np.ndarray) -> list:
        """Near-far bucket widths scaled by the batch's mean edge weight (a multiple of the
        typical edge keeps a few hops per bucket)."""
        ch = np.asarray(changes)
        live = ch[(ch["op"] == 0) | (ch["op"] == 1)] if len(ch) else ch
        wbar = float(np.mean(live["w"])) if len(live) else 0.0
        if wbar <= 0:
            return []
        return [{"delta": max(1, int(round(f * wbar)))} for f in (8.0, 96.0)]

    def tune(self, graph: Graph, changes: np.ndarray, force: bool = False) -> dict:
        """Picks the fastest candidate for (graph, changes), sets it on the graph and returns
        {"key", "opts", "ms", "trials"}; a cached class is applied without timing."""
        info = graph.info()
        key = size_class(info["n"], info["entries"], len(changes))
        base = graph.get_opts()
        if not force and key in self.cache:
            best = self.cache[key]
            graph.set_opts(self._apply(base, best["opts"]))
            return {"key": key, "opts": best["opts"], "ms": best["ms"], "trials": [], "cached": True}
        graph.snapshot()
        trials = []
        cands = list(self.candidates)
        if self.candidates is CANDIDATES:
            cands += self.near_far_candidates(changes)
        for cand in cands:
            o = self._apply(base, cand)
            try:
                graph.set_opts(o)
            except Exception:  # a candidate the device cannot run (occupancy)
                continue
            times = []
            for _ in range(self.reps):
                graph.restore()
                st = graph.apply_batch(changes)
                times.append(st.t_total_ms)
            trials.append((min(times), {f: getattr(o, f) for f in TUNED_FIELDS}))
        graph.restore()
        trials.sort(key=lambda t: t[0])
        best_ms, best = trials[0]
        graph.set_opts(self._apply(base, best))
        self.cache[key] = {"opts": best, "ms": best_ms}
        self.save()
        return {"key": key, "opts": best, "ms": best_ms, "trials": trials, "cached": False}
