"""Batching layer: many independent graphs in one device graph store, updated by one launch.

A thin binding of the native pool (`dsssp_pool_*` in include/dsssp.h, csrc/serve.cpp).  The
graphs are laid out side by side in one vertex id space (graph i owns ids [offset[i],
offset[i] + n_i)), so the store is the disjoint union of the graphs and every graph is a
separate connected part with its own source.  A set of change batches -- at most one per
graph -- becomes one change batch of the union, applied by one run of the engine's batch
kernels and one persistent update kernel.  The kernels treat every vertex that is its own
parent as a root, so each graph keeps its own tree, and the update of one graph never reads
another graph's data: the result per graph equals applying its batch alone (distances
bit-exact, parents a valid tree).

No counterpart in the reference, which updates one graph per process run.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import CHANGE_DTYPE, Graph, Opts, Stats, _check, _lib, default_opts

_P = C.c_void_p


def _ptrs(arrays):
    """A C array of the arrays' data pointers (NULL for an empty one)."""
    return (C.c_void_p * max(1, len(arrays)))(*[a.ctypes.data if len(a) else None for a in arrays])


def _batch_args(batches):
    """(count, graph ids, batch pointers, sizes, keep-alive list) for the native calls."""
    ids, arrs = [], []
    for i, ch in batches:
        ids.append(int(i))
        arrs.append(np.ascontiguousarray(ch, CHANGE_DTYPE))
    g = np.asarray(ids, np.int32)
    sizes = np.asarray([len(a) for a in arrs], np.int64)
    return len(arrs), g, _ptrs(arrs), sizes, arrs


class _PoolGraph(Graph):
    """The pool's engine graph; owned by the pool (closing it is a no-op)."""

    def __init__(self, handle: int, n: int):  # noqa: D401 - no edge arrays: the pool built it
        self._h = _P(handle)
        self.n = n

    def close(self) -> None:
        pass


class GraphPool:
    def __init__(self, graphs, opts: Opts | None = None, reserve_vertices: int = 0, **kw):
        """graphs: sequence of (n_i, u_i, v_i, w_i) edge lists with local vertex ids;
        reserve_vertices: spare ids for graphs added later (add_graph)."""
        n = np.asarray([int(g[0]) for g in graphs], np.int32)
        us = [np.ascontiguousarray(g[1], np.int32) for g in graphs]
        vs = [np.ascontiguousarray(g[2], np.int32) for g in graphs]
        ws = [np.ascontiguousarray(g[3], np.int32) for g in graphs]
        m = np.asarray([len(a) for a in us], np.int64)
        if len(n) == 0 and reserve_vertices <= 0:
            raise ValueError("a pool needs at least one graph or a vertex reserve")
        o = opts if opts is not None else default_opts(**kw)
        h = _P()
        _check(_lib.dsssp_pool_create_reserved(len(n), n.ctypes.data, m.ctypes.data, _ptrs(us), _ptrs(vs),
                                               _ptrs(ws), int(reserve_vertices), C.byref(o), C.byref(h)),
               "pool_create")
        self._h = h
        self.sizes = n.astype(np.int64)
        self.offsets = np.empty(len(n) + 1, np.int64)
        _check(_lib.dsssp_pool_offsets(h, self.offsets.ctypes.data), "pool_offsets")
        cap = C.c_int64()
        _check(_lib.dsssp_pool_capacity(h, C.byref(cap), None, None), "pool_capacity")
        self.n = int(cap.value)
        self.edges = [int(x) for x in m]
        self.graph = _PoolGraph(_lib.dsssp_pool_graph(h), self.n)

    def __len__(self) -> int:
        return len(self.sizes)

    def add_graph(self, n: int, u, v, w, src: int = 0) -> int:
        """A graph in free reserved ids: its tree is built on the device from its edges (the
        other graphs are untouched).  Returns its index."""
        u = np.ascontiguousarray(u, np.int32)
        v = np.ascontiguousarray(v, np.int32)
        w = np.ascontiguousarray(w, np.int32)
        gi = C.c_int32()
        _check(_lib.dsssp_pool_add_graph(self._h, int(n), len(u), u.ctypes.data if len(u) else None,
                                         v.ctypes.data if len(v) else None, w.ctypes.data if len(w) else None,
                                         int(src), C.byref(gi)), "pool_add_graph")
        self.sizes = np.append(self.sizes, int(n))
        self.edges.append(len(u))
        return gi.value

    def remove_graph(self, graph: int) -> None:
        _check(_lib.dsssp_pool_remove_graph(self._h, int(graph)), "pool_remove_graph")
        self.sizes[graph] = 0

    def graph_range(self, graph: int) -> tuple[int, int]:
        first, n = C.c_int64(), C.c_int32()
        _check(_lib.dsssp_pool_graph_range(self._h, int(graph), C.byref(first), C.byref(n)), "pool_graph_range")
        return first.value, n.value

    def capacity(self) -> dict:
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        _check(_lib.dsssp_pool_capacity(self._h, C.byref(a), C.byref(b), C.byref(c)), "pool_capacity")
        return {"vertices": a.value, "free": b.value, "largest_free": c.value}

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            _lib.dsssp_pool_destroy(self._h)
            self._h = _P()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

    # ---- trees -------------------------------------------------------------------------------

    def tree_compute(self, sources) -> Stats:
        """sources[i] = local source of graph i."""
        src = np.ascontiguousarray(sources, np.int32)
        if len(src) != len(self):
            raise ValueError("one source per graph")
        st = Stats()
        _check(_lib.dsssp_pool_tree_compute(self._h, src.ctypes.data, C.byref(st)), "pool_tree_compute")
        return st

    def forest_load(self, trees) -> None:
        """trees[i] = (parent_i, dist_i) with local ids (parent -1 = unreachable)."""
        par = [np.ascontiguousarray(p, np.int32) for p, _ in trees]
        dist = [np.ascontiguousarray(d, np.int64) for _, d in trees]
        if len(par) != len(self) or any(len(p) != s for p, s in zip(par, self.sizes)):
            raise ValueError("one tree of n_i entries per graph")
        _check(_lib.dsssp_pool_forest_load(self._h, _ptrs(par), _ptrs(dist)), "pool_forest_load")

    def tree_read(self, which=None):
        """Trees with local ids: a list of (parent, dist), or one tree for graph `which`."""
        out = []
        for i in (range(len(self)) if which is None else [which]):
            if self.sizes[i] == 0:  # removed
                out.append((np.zeros(0, np.int32), np.zeros(0, np.int64)))
                continue
            p = np.empty(int(self.sizes[i]), np.int32)
            d = np.empty(int(self.sizes[i]), np.int64)
            _check(_lib.dsssp_pool_tree_read(self._h, int(i), p.ctypes.data, d.ctypes.data), "pool_tree_read")
            out.append((p, d))
        return out if which is None else out[0]

    # ---- batches -----------------------------------------------------------------------------

    def union_batch(self, batches) -> np.ndarray:
        """batches: sequence of (graph index, change records with local ids); at most one batch
        per graph (two batches of one graph in one union would not equal applying them one
        after the other).  Returns the union's records (ids of the pool)."""
        nb, g, ptrs, sizes, keep = _batch_args(batches)
        k = C.c_int64()
        _check(_lib.dsssp_pool_union(self._h, nb, g.ctypes.data, ptrs, sizes.ctypes.data, None, 0, C.byref(k)),
               "pool_union")
        out = np.zeros(k.value, CHANGE_DTYPE)
        _check(_lib.dsssp_pool_union(self._h, nb, g.ctypes.data, ptrs, sizes.ctypes.data,
                                     out.ctypes.data if k.value else None, k.value, C.byref(k)), "pool_union")
        del keep
        return out

    def apply(self, batches) -> Stats:
        """Applies one batch per listed graph in one launch sequence; waits for it."""
        nb, g, ptrs, sizes, keep = _batch_args(batches)
        st = Stats()
        _check(_lib.dsssp_pool_apply(self._h, nb, g.ctypes.data, ptrs, sizes.ctypes.data, C.byref(st)), "pool_apply")
        del keep
        return st

    def footprint(self) -> int:
        return int(self.graph.info()["device_bytes"])
