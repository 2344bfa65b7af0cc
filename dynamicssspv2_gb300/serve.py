"""Serving layer: resident tenant graphs, change batches applied as they arrive.

A thin binding of the native server (`dsssp_server_*`, `dsssp_submit`, `dsssp_poll` in
include/dsssp.h, csrc/serve.cpp).  It keeps the graphs and trees of its tenants resident in
HBM in one pooled graph store, admitting tenants in order while their estimated device
footprint fits the memory budget.  Requests -- (arrival time, tenant, change batch) -- are
served with continuous batching by a native worker thread: whenever the device is free,
every tenant with a waiting request contributes its oldest request to the next epoch, and
the epoch's requests run together in one launch sequence (their work overlaps on the
device).  A tenant never has two requests in one epoch, so each tenant sees its batches
applied one after another in arrival order, and each result equals applying that batch
alone (distances bit-exact; parents a valid tree, possibly another one on ties).  Requests
that arrive while an epoch runs wait for the next one; requests for tenants that were not
admitted are refused, and a request whose batch names a vertex outside its tenant's graph or
inserts a negative weight fails on arrival (`error` says why) without touching the epoch it
would have joined.

Tenants that do not fit the memory budget wait, with their vertex ids reserved, and are
admitted when a removal frees memory; tenants can be added (`add_tenant`) and removed
(`remove_tenant`) while the server runs.  A new tenant's tree is built on the device from its
edges without touching the others.  An epoch whose update kernel fails (a device wait that
times out, for instance) is recovered by recomputing the trees on the device: its requests are
served with `recomputed` set and every tenant's tree stays exact.

Storage upkeep runs between epochs, only while no request waits: when the store's tombstoned
entries exceed `compact_dead_frac` of its live entries, or the spare region that overflowing
rows move into is more than `compact_spare_frac` used, the store is compacted (tombstones
dropped, rows re-sorted, full slack restored) so later batches keep finding slack.

No counterpart in the reference, which applies one batch per process run.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import (CHANGE_DTYPE, REFUSED, TENANT_ADMITTED, W_RECOMPUTED, RequestInfo, ServerOpts, _check, _lib,
               default_opts)
from .pool import _ptrs


def estimate_footprint(n: int, m: int, slack_pct: int = 25, slack_min: int = 4) -> int:
    """Device bytes the engine needs for a graph of n vertices and m undirected edges."""
    return int(_lib.dsssp_estimate_footprint(int(n), int(m), int(slack_pct), int(slack_min)))


@dataclass
class Tenant:
    name: str
    n: int
    u: np.ndarray
    v: np.ndarray
    w: np.ndarray
    src: int = 0


@dataclass
class Request:
    tenant: int
    arrival: float  # seconds from the start of serve()
    changes: np.ndarray
    rid: int = -1
    # filled in by the server
    epoch: int = -1
    start: float = float("nan")
    done: float = float("nan")
    refused: bool = False
    recomputed: bool = False  # served by an epoch recovered by recomputing the trees
    error: str | None = None
    result: tuple | None = field(default=None, repr=False)

    @property
    def latency(self) -> float:
        return self.done - self.arrival


class Server:
    def __init__(self, tenants, memory_budget: int | None = None, max_epoch_requests: int | None = None,
                 compact_dead_frac: float | None = 0.25, compact_spare_frac: float = 0.75,
                 reserve_vertices: int = 0, tune_cache: str | None = None, **opts):
        self.tenants = list(tenants)
        o = default_opts(**opts)
        self._slack = (o.slack_pct, o.slack_min)
        self.footprints = [estimate_footprint(t.n, len(t.u), o.slack_pct, o.slack_min) for t in self.tenants]
        so = ServerOpts()
        _lib.dsssp_default_server_opts(C.byref(so))
        so.memory_budget = int(memory_budget or 0)
        so.max_epoch_requests = int(max_epoch_requests or 0)
        so.compact_dead_frac = -1.0 if compact_dead_frac is None else float(compact_dead_frac)
        so.compact_spare_frac = float(compact_spare_frac)
        so.reserve_vertices = int(reserve_vertices)
        self._tune_cache = str(tune_cache).encode() if tune_cache else None  # kept alive for the call
        so.tune_cache = self._tune_cache
        n = np.asarray([t.n for t in self.tenants], np.int32)
        us = [np.ascontiguousarray(t.u, np.int32) for t in self.tenants]
        vs = [np.ascontiguousarray(t.v, np.int32) for t in self.tenants]
        ws = [np.ascontiguousarray(t.w, np.int32) for t in self.tenants]
        m = np.asarray([len(a) for a in us], np.int64)
        src = np.asarray([t.src for t in self.tenants], np.int32)
        h = C.c_void_p()
        _check(_lib.dsssp_server_create(len(n), n.ctypes.data, m.ctypes.data, _ptrs(us), _ptrs(vs), _ptrs(ws),
                                        src.ctypes.data, C.byref(so), C.byref(o), C.byref(h)), "server_create")
        self._h = h
        self.reserved = sum(self.footprints[t] for t in self.admitted)

    @property
    def admitted(self) -> list[int]:
        """Tenants in the pool now (in tenant order); after close, those at close."""
        if not (getattr(self, "_h", None) and self._h.value):
            return list(getattr(self, "_admitted_final", []))
        return [t for t in range(len(self.tenants)) if self.state(t) == TENANT_ADMITTED]

    @property
    def slot(self) -> dict:
        return {t: _lib.dsssp_server_slot(self._h, t) for t in self.admitted}

    def state(self, tenant: int) -> int:
        """TENANT_WAITING, TENANT_ADMITTED or TENANT_REMOVED."""
        return _check(_lib.dsssp_server_tenant_state(self._h, int(tenant)), "server_tenant_state")

    def add_tenant(self, tenant: Tenant) -> int:
        """Adds a tenant while the server runs: admitted at once when its footprint fits the
        budget and free vertex ids exist (its tree is built on the device), else it waits for
        a removal to free memory.  Returns its tenant id."""
        u = np.ascontiguousarray(tenant.u, np.int32)
        v = np.ascontiguousarray(tenant.v, np.int32)
        w = np.ascontiguousarray(tenant.w, np.int32)
        t = C.c_int32()
        _check(_lib.dsssp_server_add_tenant(self._h, int(tenant.n), len(u), u.ctypes.data if len(u) else None,
                                            v.ctypes.data if len(v) else None, w.ctypes.data if len(w) else None,
                                            int(tenant.src), C.byref(t)), "server_add_tenant")
        assert t.value == len(self.tenants)
        self.tenants.append(tenant)
        self.footprints.append(estimate_footprint(tenant.n, len(u), *self._slack))
        return t.value

    def remove_tenant(self, tenant: int) -> None:
        """Removes a tenant after the running epoch: its queued requests are refused, its memory
        is released and waiting tenants that now fit are admitted."""
        _check(_lib.dsssp_server_remove_tenant(self._h, int(tenant)), "server_remove_tenant")

    @property
    def recovered_epochs(self) -> int:
        e = C.c_int64()
        _check(_lib.dsssp_server_recovered_epochs(self._h, C.byref(e)), "server_recovered_epochs")
        return e.value

    def debug_set(self, what: int, value: int) -> None:
        """Failure-detection test hooks on the pool's graph, applied between epochs."""
        _check(_lib.dsssp_server_debug_set(self._h, int(what), int(value)), "server_debug_set")

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._final = self._info()  # counters stay readable after close
            self._admitted_final = self.admitted
            _lib.dsssp_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

    def _info(self):
        if not (getattr(self, "_h", None) and self._h.value):
            return self._final
        e, c, pend = C.c_int64(), C.c_int64(), C.c_int64()
        ms = C.c_double()
        _check(_lib.dsssp_server_info(self._h, C.byref(e), C.byref(c), C.byref(ms), C.byref(pend)), "server_info")
        return e.value, c.value, ms.value, pend.value

    @property
    def epochs(self) -> int:
        return self._info()[0]

    @property
    def compactions(self) -> int:
        return self._info()[1]

    def validate(self) -> dict:
        """Device certificate of every admitted tenant's tree: {violations, roots}."""
        bad, roots = C.c_int64(), C.c_int64()
        _check(_lib.dsssp_server_validate(self._h, C.byref(bad), C.byref(roots)), "server_validate")
        return {"violations": bad.value, "roots": roots.value}

    def tree(self, tenant: int):
        t = self.tenants[tenant]
        p = np.empty(t.n, np.int32)
        d = np.empty(t.n, np.int64)
        _check(_lib.dsssp_server_tree_read(self._h, int(tenant), p.ctypes.data, d.ctypes.data), "server_tree_read")
        return p, d

    def serve(self, requests, record: bool = False, realtime: bool = True, timeout_s: float = 600.0):
        """Submits the requests (sorted by arrival) and returns them with epoch, start and done
        times (seconds, on the arrival clock) and latency filled in.  realtime submits each
        request at its arrival time; realtime=False submits all at once (a saturated server)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        for i, r in enumerate(reqs):
            if r.rid < 0:
                r.rid = i
        _check(_lib.dsssp_server_set_record(self._h, 1 if record else 0), "server_set_record")
        arrays = [np.ascontiguousarray(r.changes, CHANGE_DTYPE) for r in reqs]
        by_id = {}
        if realtime:
            t0 = time.perf_counter()
            for r, a in zip(reqs, arrays):
                while True:
                    wait = r.arrival - (time.perf_counter() - t0)
                    if wait <= 0:
                        break
                    if wait > 0.0005:
                        time.sleep(min(wait - 0.0002, 0.002))
                rid = C.c_int64()
                _check(_lib.dsssp_submit(self._h, int(r.tenant), a.ctypes.data if len(a) else None, len(a),
                                         C.byref(rid)), "submit")
                by_id[rid.value] = r
        elif reqs:
            ten = np.asarray([r.tenant for r in reqs], np.int32)
            sizes = np.asarray([len(a) for a in arrays], np.int64)
            ids = np.empty(len(reqs), np.int64)
            _check(_lib.dsssp_submit_many(self._h, len(reqs), ten.ctypes.data, _ptrs(arrays), sizes.ctypes.data,
                                          ids.ctypes.data), "submit_many")
            by_id = {int(i): r for i, r in zip(ids, reqs)}
        _check(_lib.dsssp_server_drain(self._h, int(timeout_s * 1000)), "server_drain")
        buf = (RequestInfo * 256)()
        cnt = C.c_int32()
        left = len(by_id)
        while left:
            _check(_lib.dsssp_poll(self._h, buf, 256, 100, C.byref(cnt)), "poll")
            for info in buf[: cnt.value]:
                r = by_id[info.id]
                left -= 1
                # the native clock starts with the server: keep each request on its own
                # arrival clock and carry over the native intervals
                r.epoch = int(info.epoch)
                r.start = r.arrival + (info.start_us - info.arrival_us) * 1e-6
                r.done = r.arrival + (info.done_us - info.arrival_us) * 1e-6
                r.refused = info.status == REFUSED
                r.recomputed = info.status == W_RECOMPUTED
                r.error = None if info.status in (0, REFUSED, W_RECOMPUTED) else info.error.decode(errors="replace")
                if record and info.status in (0, W_RECOMPUTED):
                    t = self.tenants[r.tenant]
                    p = np.empty(t.n, np.int32)
                    d = np.empty(t.n, np.int64)
                    _check(_lib.dsssp_server_result(self._h, info.id, p.ctypes.data, d.ctypes.data), "server_result")
                    r.result = (p, d)
        return reqs


def summarize(reqs) -> dict:
    served = [r for r in reqs if not r.refused and r.error is None]
    lat = np.array([r.latency for r in served]) if served else np.zeros(0)
    changes = sum(len(r.changes) for r in served)
    span = (max(r.done for r in served) - min(r.arrival for r in served)) if served else 0.0
    return {
        "requests": len(reqs),
        "served": len(served),
        "refused": sum(1 for r in reqs if r.refused),
        "recomputed": sum(1 for r in reqs if r.recomputed),
        "failed": sum(1 for r in reqs if r.error is not None),
        "changes": int(changes),
        "span_s": span,
        "change_edges_per_s": changes / span if span > 0 else 0.0,
        "p50_ms": float(np.percentile(lat, 50) * 1e3) if len(lat) else None,
        "p99_ms": float(np.percentile(lat, 99) * 1e3) if len(lat) else None,
        "mean_ms": float(lat.mean() * 1e3) if len(lat) else None,
        "epochs": len({r.epoch for r in served}),
        "mean_requests_per_epoch": len(served) / max(1, len({r.epoch for r in served})),
    }


def random_batch(rng: np.random.Generator, tenant: Tenant, size: int, ins_frac: float = 0.5,
                 wlo: int = 1, whi: int = 100) -> np.ndarray:
    """A change batch for a tenant: insertions of random vertex pairs, deletions of random
    lines of the tenant's base edge list (possibly already deleted: then a no-op)."""
    n_ins = int(round(size * ins_frac))
    n_del = min(size - n_ins, len(tenant.u))
    ch = np.zeros(n_ins + n_del, CHANGE_DTYPE)
    a = rng.integers(0, tenant.n, n_ins)
    b = rng.integers(0, tenant.n, n_ins)
    b = np.where(a == b, (b + 1) % tenant.n, b)
    ch["u"][:n_ins], ch["v"][:n_ins] = a, b
    ch["w"][:n_ins] = rng.integers(wlo, whi + 1, n_ins)
    ch["op"][:n_ins] = 1
    idx = rng.choice(len(tenant.u), n_del, replace=False) if n_del else np.zeros(0, np.int64)
    ch["u"][n_ins:], ch["v"][n_ins:], ch["w"][n_ins:] = tenant.u[idx], tenant.v[idx], tenant.w[idx]
    ch["op"][n_ins:] = 0
    return ch[rng.permutation(len(ch))]
