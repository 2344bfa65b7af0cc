"""Batching layer: many independent graphs in one device graph store, updated by one launch.

The graphs are laid out side by side in one vertex id space (graph i owns ids
[offset[i], offset[i] + n_i)), so the store is the disjoint union of the graphs and every
graph is a separate connected part with its own source.  A set of change batches -- at most
one per graph -- becomes one change batch of the union, applied by one run of the engine's
batch kernels and one persistent update kernel.  The kernels treat every vertex that is its
own parent as a root, so each graph keeps its own tree, and the update of one graph never
reads another graph's data: the result per graph equals applying its batch alone
(distances bit-exact, parents a valid tree).

No counterpart in the reference, which updates one graph per process run.
"""
from __future__ import annotations

import numpy as np

from . import CHANGE_DTYPE, Graph, Opts, Stats, default_opts


class GraphPool:
    def __init__(self, graphs, opts: Opts | None = None, **kw):
        """graphs: sequence of (n_i, u_i, v_i, w_i) edge lists with local vertex ids."""
        sizes = np.array([int(g[0]) for g in graphs], np.int64)
        if len(sizes) == 0 or (sizes <= 0).any():
            raise ValueError("every graph needs at least one vertex")
        self.sizes = sizes
        self.offsets = np.concatenate([[0], np.cumsum(sizes)])
        if self.offsets[-1] >= 2**31 - 16:
            raise ValueError("the pool's vertex count must stay below 2^31")
        us, vs, ws = [], [], []
        for i, (n, u, v, w) in enumerate(graphs):
            off = self.offsets[i]
            u = np.asarray(u, np.int64)
            v = np.asarray(v, np.int64)
            if len(u) and (u.min() < 0 or u.max() >= n or v.min() < 0 or v.max() >= n):
                raise ValueError(f"graph {i}: vertex id outside 0..{n - 1}")
            us.append((u + off).astype(np.int32))
            vs.append((v + off).astype(np.int32))
            ws.append(np.asarray(w, np.int32))
        self.n = int(self.offsets[-1])
        self.edges = [len(g[1]) for g in graphs]
        self.graph = Graph(self.n, np.concatenate(us), np.concatenate(vs), np.concatenate(ws),
                           opts if opts is not None else default_opts(**kw))

    def __len__(self) -> int:
        return len(self.sizes)

    def close(self) -> None:
        self.graph.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- trees -------------------------------------------------------------------------------

    def tree_compute(self, sources) -> Stats:
        """sources[i] = local source of graph i."""
        src = np.asarray(sources, np.int64)
        if len(src) != len(self) or (src < 0).any() or (src >= self.sizes).any():
            raise ValueError("one in-range source per graph")
        return self.graph.tree_compute_multi((src + self.offsets[:-1]).astype(np.int32))

    def forest_load(self, trees) -> None:
        """trees[i] = (parent_i, dist_i) with local ids (parent -1 = unreachable)."""
        parent = np.empty(self.n, np.int32)
        dist = np.empty(self.n, np.int64)
        for i, (p, d) in enumerate(trees):
            a, b = self.offsets[i], self.offsets[i + 1]
            p = np.asarray(p, np.int64)
            parent[a:b] = np.where(p < 0, -1, p + a)
            dist[a:b] = d
        self.graph.forest_load(parent, dist)

    def tree_read(self, which=None):
        """Trees with local ids: a list of (parent, dist), or one tree for graph `which`."""
        parent, dist = self.graph.tree_read()
        out = []
        idx = range(len(self)) if which is None else [which]
        for i in idx:
            a, b = self.offsets[i], self.offsets[i + 1]
            p = parent[a:b].astype(np.int64)
            out.append((np.where(p < 0, -1, p - a).astype(np.int32), dist[a:b].copy()))
        return out if which is None else out[0]

    # ---- batches -----------------------------------------------------------------------------

    def union_batch(self, batches) -> np.ndarray:
        """batches: sequence of (graph index, change records with local ids); at most one
        batch per graph (two batches of one graph in one union would not equal applying them
        one after the other)."""
        seen = set()
        parts = []
        for i, ch in batches:
            i = int(i)
            if i in seen:
                raise ValueError(f"graph {i} has two batches in one union")
            if not 0 <= i < len(self):
                raise ValueError(f"no graph {i}")
            seen.add(i)
            ch = np.asarray(ch, CHANGE_DTYPE)
            live = (ch["op"] == 0) | (ch["op"] == 1)
            n = self.sizes[i]
            if ((ch["u"][live] < 0) | (ch["u"][live] >= n) | (ch["v"][live] < 0) | (ch["v"][live] >= n)).any():
                raise ValueError(f"graph {i}: change names a vertex outside 0..{n - 1}")
            shifted = ch.copy()
            shifted["u"] = ch["u"] + self.offsets[i]
            shifted["v"] = ch["v"] + self.offsets[i]
            parts.append(shifted)
        return np.concatenate(parts) if parts else np.zeros(0, CHANGE_DTYPE)

    def apply(self, batches) -> Stats:
        """Applies one batch per listed graph in one launch sequence; waits for it."""
        return self.graph.apply_batch(self.union_batch(batches))

    def footprint(self) -> int:
        return int(self.graph.info()["device_bytes"])
