"""Serving layer: resident tenant graphs, change batches applied as they arrive.

A Server keeps the graphs and trees of its tenants resident in HBM in one pooled graph store
(`GraphPool`), admitting tenants in order while their estimated device footprint fits the
memory budget.  Requests -- (arrival time, tenant, change batch) -- are served with
continuous batching: whenever the device is free, every tenant with a waiting request
contributes its oldest request to the next epoch, and the epoch's requests run together in
one launch sequence (their work overlaps on the device).  A tenant never has two requests
in one epoch, so each tenant sees its batches applied one after another in arrival order,
and each result equals applying that batch alone (distances bit-exact; parents a valid
tree, possibly another one on ties).  Requests that arrive while an epoch runs wait for the
next one; requests for tenants that were not admitted are refused, and a request whose
batch names a vertex outside its tenant's graph or inserts a negative weight fails on
arrival (`error` says why) without touching the epoch it would have joined.

Storage upkeep runs between epochs, only while no request waits: when the store's tombstoned
entries exceed `compact_dead_frac` of its live entries, or the spare region that overflowing
rows move into is more than `compact_spare_frac` used, the store is compacted (tombstones
dropped, rows re-sorted, full slack restored) so later batches keep finding slack.

No counterpart in the reference, which applies one batch per process run.
"""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass, field

import numpy as np

from . import CHANGE_DTYPE
from .pool import GraphPool

# Device bytes per vertex and per adjacency slot of the engine's graph store: state 8, row
# descriptor 16, sorted-prefix length 4, three tags 12, cut-off root list 4; per slot the
# entry 8 and the twin 4; work lists: three lists of thread items (8 B per slot / te + per
# vertex) and three of CTA items; plus a snapshot-free margin.
_BYTES_PER_VERTEX = 8 + 16 + 4 + 12 + 4 + 3 * 8
_BYTES_PER_SLOT = 8 + 4 + 3 * 8 / 4


def estimate_footprint(n: int, m: int, slack_pct: int = 25, slack_min: int = 4) -> int:
    """Device bytes the engine needs for a graph of n vertices and m undirected edges."""
    slots = 2 * m * (1 + slack_pct / 100.0) + n * slack_min
    return int(n * _BYTES_PER_VERTEX + slots * _BYTES_PER_SLOT + (1 << 20))


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
    error: str | None = None
    result: tuple | None = field(default=None, repr=False)

    @property
    def latency(self) -> float:
        return self.done - self.arrival


class Server:
    def __init__(self, tenants, memory_budget: int | None = None, max_epoch_requests: int | None = None,
                 compact_dead_frac: float | None = 0.25, compact_spare_frac: float = 0.75, **opts):
        self.tenants = list(tenants)
        slack_pct = opts.get("slack_pct", 25)
        slack_min = opts.get("slack_min", 4)
        self.footprints = [estimate_footprint(t.n, len(t.u), slack_pct, slack_min) for t in self.tenants]
        self.admitted = []
        used = 0
        for i, fp in enumerate(self.footprints):
            if memory_budget is None or used + fp <= memory_budget:
                self.admitted.append(i)
                used += fp
        self.reserved = used
        self.slot = {t: j for j, t in enumerate(self.admitted)}  # tenant index -> pool index
        self.max_epoch_requests = max_epoch_requests
        self.pool = None
        if self.admitted:
            ts = [self.tenants[i] for i in self.admitted]
            self.pool = GraphPool([(t.n, t.u, t.v, t.w) for t in ts], **opts)
            self.pool.tree_compute([t.src for t in ts])
        self.epochs = 0
        self.compact_dead_frac = compact_dead_frac
        self.compact_spare_frac = compact_spare_frac
        self.compactions = 0
        self.compact_ms = []

    def close(self) -> None:
        if self.pool is not None:
            self.pool.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def needs_compaction(self) -> bool:
        if self.pool is None or self.compact_dead_frac is None:
            return False
        h = self.pool.graph.health()
        if h["dead"] > self.compact_dead_frac * max(1, h["live"]):
            return True
        return h["spare_total"] > 0 and h["spare_used"] > self.compact_spare_frac * h["spare_total"]

    def upkeep(self) -> bool:
        """Compacts the store if it needs it; call only while no request waits."""
        if not self.needs_compaction():
            return False
        t = time.perf_counter()
        self.pool.graph.compact()
        self.compact_ms.append((time.perf_counter() - t) * 1e3)
        self.compactions += 1
        return True

    def check(self, r: Request) -> str | None:
        """Why the request's batch cannot be applied to its tenant, or None."""
        ch = np.asarray(r.changes, CHANGE_DTYPE)
        live = (ch["op"] == 0) | (ch["op"] == 1)
        n = self.tenants[r.tenant].n
        cu, cv = ch["u"][live], ch["v"][live]
        if ((cu < 0) | (cu >= n) | (cv < 0) | (cv >= n)).any():
            return f"a change names a vertex outside 0..{n - 1}"
        if ((ch["op"] == 1) & (ch["w"] < 0)).any():
            return "an insertion has a negative weight"
        return None

    def tree(self, tenant: int):
        return self.pool.tree_read(self.slot[tenant])

    def serve(self, requests, record: bool = False, realtime: bool = True):
        """Serves the requests (sorted by arrival); returns them with epoch, done time and
        latency filled in.  realtime=False ignores arrival gaps (saturated server)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        for i, r in enumerate(reqs):
            if r.rid < 0:
                r.rid = i
        queues = collections.defaultdict(collections.deque)
        nxt = 0
        t0 = time.perf_counter()
        clock = lambda: time.perf_counter() - t0  # noqa: E731
        pending = 0
        while nxt < len(reqs) or pending:
            now = clock() if realtime else float("inf")
            while nxt < len(reqs) and reqs[nxt].arrival <= now:
                r = reqs[nxt]
                nxt += 1
                if r.tenant not in self.slot:
                    r.refused = True
                    r.done = r.start = r.arrival
                    continue
                r.error = self.check(r)
                if r.error is not None:
                    r.done = r.start = r.arrival
                    continue
                queues[r.tenant].append(r)
                pending += 1
            if pending == 0:
                self.upkeep()  # idle: storage upkeep is off the latency path
                if nxt < len(reqs):
                    wait = reqs[nxt].arrival - clock()
                    if wait > 0:
                        time.sleep(min(wait, 0.002) if wait > 0.0005 else 0)
                continue
            epoch = []
            for t in sorted(queues, key=lambda t: queues[t][0].arrival if queues[t] else float("inf")):
                if queues[t]:
                    epoch.append(queues[t].popleft())
                    if self.max_epoch_requests and len(epoch) >= self.max_epoch_requests:
                        break
            pending -= len(epoch)
            start = clock()
            self.pool.apply([(self.slot[r.tenant], r.changes) for r in epoch])
            done = clock()
            for r in epoch:
                r.epoch = self.epochs
                r.start = start
                r.done = done
                if record:
                    r.result = self.pool.tree_read(self.slot[r.tenant])
            self.epochs += 1
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
