"""Randomized parity soak: random graph shapes (Erdos-Renyi, RMAT, long paths with chords,
hub stars, grids with diagonals, parallel edges with self-loops and zero weights, several
components), random option sets and chains of one to four random batches (uniform changes,
deleted tree edges, ignored op codes, absent deletions, insert-then-delete pairs, lighter
duplicates of existing edges, empty batches), with compaction and snapshots in between.  Every
tree is checked against the oracle's Dijkstra on the updated graph (distances bit-exact,
parents a valid shortest-path tree), the device certificate, the changed-entries read and the
32-bit read.  DSSSP_SOAK_CASES sets the number of cases (default 600, a few seconds)."""
import os

import numpy as np
import pytest

import dynamicssspv2_gb300 as D
from dynamicssspv2_gb300.pool import GraphPool
from oracle import pyoracle as O
from tests.common import check_against_oracle, lines_after

pytestmark = pytest.mark.gpu

OPT_CHOICES = {
    "bfs_levels": [0, 1, 2, 3, 48],
    "small_deg": [4, 8, 16, 64],
    "large_deg": [4, 16, 64, 256, 1 << 20],
    "chunk": [32, 128, 1024],
    "delta": [-1, -1, 0, 1, 7, 50, 400],
    "block": [64, 128, 256],
    "ctas_per_sm": [0, 1, 2],
    "launch_graph": [0, 1],
    "warp_agg": [0, 0, 1],
    "solo_waves": [0, 1, 2, 16],
    "group_ctas": [0, 0, 2, 4],
    "group_waves": [2, 16],
    "timing": [0, 1, 2],
    "auto_rounds": [4, 256],
}
SLACKS = [{}, {"slack_pct": 0, "slack_min": 0, "spare_pct": 300}, {"slack_pct": 0, "slack_min": 0, "spare_pct": 0},
          {"slack_pct": 5, "slack_min": 1, "spare_pct": 2}]


def rand_opts(rng):
    o = {}
    for k, vals in OPT_CHOICES.items():
        if rng.random() < 0.35:
            o[k] = vals[rng.integers(len(vals))]
    o.update(SLACKS[rng.integers(len(SLACKS))])
    if o.get("large_deg", 256) < o.get("small_deg", 4):
        o["large_deg"] = o.get("small_deg", 4)
    return o


def rand_graph(rng, seed):
    kind = ["er", "rmat", "path", "star", "grid", "multi", "components"][rng.integers(7)]
    wlo = int(rng.choice([0, 1, 1, 1]))
    whi = int(rng.choice([3, 50, 1000]))
    if kind == "er":
        n = int(rng.integers(2, 3000))
        m = int(min(n * (n - 1) // 2, n * rng.uniform(0.5, 8)))
        u, v, w = D.gen_er(n, max(m, 1), wlo, whi, seed) if n > 1 else (np.zeros(0, np.int32),) * 3
    elif kind == "rmat":
        scale = int(rng.integers(4, 12))
        n = 1 << scale
        m = int(min(n * (n - 1) // 4, n * rng.uniform(1, 8)))
        u, v, w = D.gen_rmat(scale, max(m, 1), 0.57, 0.19, 0.19, wlo, whi, seed)
    elif kind == "path":  # deep trees: many walk levels, pointer jumping, many rounds
        n = int(rng.integers(2, 4000))
        u = np.arange(n - 1, dtype=np.int32)
        v = u + 1
        w = rng.integers(wlo, whi + 1, n - 1).astype(np.int32)
        k = int(rng.integers(0, max(1, n // 20)))
        cu, cv = rng.integers(0, n, k), rng.integers(0, n, k)
        u = np.concatenate([u, cu]).astype(np.int32)
        v = np.concatenate([v, cv]).astype(np.int32)
        w = np.concatenate([w, rng.integers(wlo, whi + 1, k)]).astype(np.int32)
    elif kind == "star":  # hubs with long rows plus chains hanging off them
        n = int(rng.integers(10, 5000))
        hubs = int(rng.integers(1, 4))
        leaves = np.arange(hubs, n)
        u = rng.integers(0, hubs, len(leaves)).astype(np.int32)
        v = leaves.astype(np.int32)
        k = int(rng.integers(0, n))
        u = np.concatenate([u, rng.integers(0, n, k)]).astype(np.int32)
        v = np.concatenate([v, rng.integers(0, n, k)]).astype(np.int32)
        w = rng.integers(wlo, whi + 1, len(u)).astype(np.int32)
    elif kind == "grid":
        r, c = int(rng.integers(2, 60)), int(rng.integers(2, 60))
        u, v, w = D.gen_grid(r, c, float(rng.uniform(0, 0.2)), int(rng.integers(0, r * c // 10 + 1)), max(wlo, 1), whi,
                             seed)
        n = r * c
    elif kind == "multi":  # parallel edges, self-loops, zero weights
        n = int(rng.integers(2, 500))
        m = int(rng.integers(1, 4 * n))
        u = rng.integers(0, n, m).astype(np.int32)
        v = rng.integers(0, n, m).astype(np.int32)
        w = rng.integers(0, 4, m).astype(np.int32)
        dup = rng.integers(0, m, m // 4)
        u, v, w = (np.concatenate([a, a[dup]]).astype(np.int32) for a in (u, v, w))
    else:  # components: several ER parts, the source in one of them
        parts, off = [], 0
        for _ in range(int(rng.integers(2, 6))):
            pn = int(rng.integers(2, 600))
            pm = int(min(pn * (pn - 1) // 2, pn * 3))
            a, b, c = D.gen_er(pn, max(pm, 1), wlo, whi, seed + off)
            parts.append((a + off, b + off, c))
            off += pn
        n = off
        u, v, w = (np.concatenate([p[i] for p in parts]).astype(np.int32) for i in range(3))
    return kind, n, np.asarray(u, np.int32), np.asarray(v, np.int32), np.asarray(w, np.int32)


def rand_batch(rng, n, u, v, w, parent, seed):
    m = len(u)
    if rng.random() < 0.04:
        return np.zeros(0, D.CHANGE_DTYPE)
    parts = []
    if m and rng.random() < 0.8:
        try:
            ch = D.gen_changes(n, u, v, w, int(rng.integers(0, max(2, m // 5))), int(rng.integers(0, max(2, m // 5))),
                               seed=seed, wlo=0 if rng.random() < 0.2 else 1, whi=int(rng.choice([3, 50, 1000])))
            parts.append(ch)
        except D.DsssspError:  # no new pairs left in a (nearly) complete graph
            pass
    # tree edges deleted on purpose (cut-offs)
    tv = np.flatnonzero((parent >= 0) & (parent != np.arange(n)))
    if len(tv):
        pick = rng.choice(tv, int(min(len(tv), rng.integers(0, 20))), replace=False)
        for x in pick:
            p = parent[x]
            hit = np.flatnonzero(((u == x) & (v == p)) | ((u == p) & (v == x)))
            if len(hit):
                j = hit[rng.integers(len(hit))]
                parts.append(D.make_changes([u[j]], [v[j]], [w[j]], [0]))
    # noise: unknown ops, absent deletions, insert-then-delete, zero-weight and duplicate inserts
    k = int(rng.integers(0, 10))
    if k:
        a = rng.integers(0, n, k)
        b = rng.integers(0, n, k)
        ww = rng.integers(0, 20, k)
        ops = rng.choice([0, 1, 1, 2, -1], k)
        parts.append(D.make_changes(a, b, ww, ops))
        ins = rng.integers(0, n, 2)
        wgt = int(rng.integers(0, 20))
        parts.append(D.make_changes([ins[0], ins[1]], [ins[1], ins[0]], [wgt, wgt], [1, 0]))
    if m and rng.random() < 0.3:
        j = rng.integers(0, m, 3)
        parts.append(D.make_changes(u[j], v[j], np.maximum(w[j] - 1, 0), [1, 1, 1]))
        parts.append(D.make_changes(u[j[:1]], v[j[:1]], w[j[:1]], [0]))
    if not parts:
        return np.zeros(0, D.CHANGE_DTYPE)
    ch = np.concatenate(parts)
    return ch[rng.permutation(len(ch))]


def one_case(seed):
    """One random graph, option set and chain of batches; raises on any mismatch."""
    rng = np.random.default_rng(seed)
    kind, n, u, v, w = rand_graph(rng, seed)
    opts = rand_opts(rng)
    src = int(rng.integers(0, n))
    try:
        g = D.Graph(n, u, v, w, **opts)
    except D.DsssspError as e:
        if e.args and "invalid dsssp_opts" in str(e):
            return "skip-opts", kind, opts
        raise
    with g:
        if rng.random() < 0.5:
            g.tree_compute(src)
        else:
            dist, parent = O.dijkstra(n, O.csr(n, u, v, w), src)
            g.tree_load(parent, dist)
        p, d = g.tree_read()
        check_against_oracle(n, u, v, w, np.zeros(0, D.CHANGE_DTYPE), src, p, d, f"{seed} {kind} initial")
        host_p, host_d = p.copy(), d.copy()
        snap = None
        for b in range(int(rng.integers(1, 5))):
            ch = rand_batch(rng, n, u, v, w, host_p, seed * 10 + b)
            if rng.random() < 0.2:
                g.snapshot()
                snap = (u, v, w, host_p.copy(), host_d.copy(), g.health(), g.info()["entries"])
            st = g.apply_batch(ch)
            p, d = g.tree_read()
            where = f"seed {seed} {kind} n={n} m={len(u)} batch {b} k={len(ch)} opts {opts}"
            assert st.recovered_from == 0, f"{where}: recovered from {st.recovered_from}: {D._lib.dsssp_last_error()}"
            check_against_oracle(n, u, v, w, ch, src, p, d, where)
            c = g.validate()
            assert c["violations"] == 0, f"{where}: certificate {c}"
            vx, pp, dd = g.tree_read_changed()
            host_p[vx], host_d[vx] = pp, dd
            assert np.array_equal(host_p, p) and np.array_equal(host_d, d), f"{where}: changed entries"
            p32, d32 = g.tree_read32()
            assert np.array_equal(p32, p) and np.array_equal(np.where(d < 0, D.UNREACHABLE32, d).astype(np.uint32), d32)
            u, v, w = lines_after(n, u, v, w, ch)
            if rng.random() < 0.2:
                g.compact()
            if snap is not None and rng.random() < 0.3:  # back to the snapshot; later batches start there
                g.restore()
                u, v, w, sp, sd, health, entries = snap
                p, d = g.tree_read()
                assert np.array_equal(p, sp) and np.array_equal(d, sd), f"{where}: restored tree"
                assert g.health() == health and g.info()["entries"] == entries, f"{where}: restored graph"
                host_p, host_d = sp.copy(), sd.copy()
    return "ok", kind, opts


CASES = int(os.environ.get("DSSSP_SOAK_CASES", "600"))
BLOCKS = 6


@pytest.mark.parametrize("block", range(BLOCKS))
def test_random_cases(block):
    per = (CASES + BLOCKS - 1) // BLOCKS
    kinds = {}
    for seed in range(block * per, min(CASES, (block + 1) * per)):
        res, kind, _ = one_case(seed)
        kinds[kind] = kinds.get(kind, 0) + (res == "ok")
    assert sum(kinds.values()) > 0


def pool_case(seed):
    """A pooled store of one to six random graphs: batches for random subsets of them in one
    launch sequence, graphs added into the vertex reserve and removed; every graph's tree
    checked against the oracle after each step, the union certified on the device."""
    rng = np.random.default_rng(1_000_000 + seed)
    graphs = [rand_graph(rng, 50 * seed + i)[1:] for i in range(int(rng.integers(1, 7)))]
    opts = rand_opts(rng)
    reserve = int(rng.choice([0, 0, 3000, 12000]))
    try:
        pool = GraphPool(graphs, reserve_vertices=reserve, **opts)
    except D.DsssspError as e:
        if "invalid dsssp_opts" in str(e):
            return "skip-opts"
        raise
    with pool:
        live = [{"n": n, "u": u, "v": v, "w": w, "src": int(rng.integers(0, n))} for n, u, v, w in graphs]
        pool.tree_compute([g["src"] for g in live])
        for step in range(int(rng.integers(1, 5))):
            where = f"pool seed {seed} step {step} opts {opts}"
            if reserve and rng.random() < 0.4:
                _, n, u, v, w = rand_graph(rng, 50 * seed + 40 + step)
                if n <= pool.capacity()["largest_free"]:
                    src = int(rng.integers(0, n))
                    assert pool.add_graph(n, u, v, w, src) == len(live)
                    live.append({"n": n, "u": u, "v": v, "w": w, "src": src})
            alive = [i for i, g in enumerate(live) if g is not None]
            if len(alive) > 1 and rng.random() < 0.2:
                gone = alive[int(rng.integers(len(alive)))]
                pool.remove_graph(gone)
                live[gone] = None
                alive.remove(gone)
            pick = [i for i in alive if rng.random() < 0.7]
            batches = []
            for i in pick:
                g = live[i]
                parent = pool.tree_read(i)[0]
                batches.append((i, rand_batch(rng, g["n"], g["u"], g["v"], g["w"], parent, 7 * seed + i)))
            if batches:
                st = pool.apply(batches)
                assert st.recovered_from == 0, f"{where}: recovered from {st.recovered_from}"
            changes = dict(batches)
            for i in alive:
                g = live[i]
                ch = changes.get(i, np.zeros(0, D.CHANGE_DTYPE))
                p, d = pool.tree_read(i)
                check_against_oracle(g["n"], g["u"], g["v"], g["w"], ch, g["src"], p, d, f"{where} graph {i}")
                g["u"], g["v"], g["w"] = lines_after(g["n"], g["u"], g["v"], g["w"], ch)
            c = pool.graph.validate()
            assert c["violations"] == 0, f"{where}: certificate {c}"
    return "ok"


def server_case(seed):
    """A server with one to five random tenants under a random memory budget: requests
    submitted at once (epochs of several tenants), tenants removed and added between the
    rounds of requests; every served request's recorded tree checked against the oracle, the
    refused ones exactly those of tenants not admitted, the trees certified on the device."""
    from dynamicssspv2_gb300 import serve as S

    rng = np.random.default_rng(2_000_000 + seed)
    tenants = []
    for i in range(int(rng.integers(1, 6))):
        _, n, u, v, w = rand_graph(rng, 60 * seed + i)
        tenants.append(S.Tenant(f"t{i}", n, u, v, w, int(rng.integers(0, n))))
    fps = [S.estimate_footprint(t.n, len(t.u)) for t in tenants]
    budget = None if rng.random() < 0.5 else int(sum(fps) * rng.uniform(0.4, 1.1))
    opts = rand_opts(rng)
    opts.pop("timing", None)
    try:
        srv = S.Server(tenants, memory_budget=budget, max_epoch_requests=[None, 1, 3][int(rng.integers(3))],
                       reserve_vertices=int(rng.choice([0, 8000])), **opts)
    except D.DsssspError as e:
        if "invalid dsssp_opts" in str(e):
            return "skip-opts"
        raise
    with srv:
        graphs = [[t.u, t.v, t.w] for t in tenants]
        for rnd in range(int(rng.integers(1, 4))):
            where = f"server seed {seed} round {rnd} opts {opts} budget {budget}"
            admitted = set(srv.admitted)
            reqs, expect = [], {}
            for j in range(int(rng.integers(1, 16))):
                t = int(rng.integers(len(srv.tenants)))
                ten = srv.tenants[t]
                if t in admitted:
                    u, v, w = expect.get(t, graphs[t])
                    parent = O.dijkstra(ten.n, O.csr(ten.n, u, v, w), ten.src)[1]
                    ch = rand_batch(rng, ten.n, u, v, w, parent, 9 * seed + 31 * rnd + j)
                    expect[t] = list(lines_after(ten.n, u, v, w, ch))
                else:
                    ch = D.make_changes([0], [0], [1], [1])
                reqs.append(S.Request(t, arrival=0.0, changes=ch))
            for r in srv.serve(reqs, record=True, realtime=False):
                assert r.error is None and not r.recomputed, f"{where}: request {r.rid}: {r.error}"
                assert r.refused == (r.tenant not in admitted), f"{where}: request {r.rid} refused={r.refused}"
                if r.refused:
                    continue
                ten = srv.tenants[r.tenant]
                u, v, w = graphs[r.tenant]
                check_against_oracle(ten.n, u, v, w, r.changes, ten.src, *r.result, f"{where} request {r.rid}")
                graphs[r.tenant] = list(lines_after(ten.n, u, v, w, r.changes))
            c = srv.validate()
            assert c["violations"] == 0, f"{where}: certificate {c}"
            if len(admitted) > 1 and rng.random() < 0.3:
                srv.remove_tenant(sorted(admitted)[int(rng.integers(len(admitted)))])
            if rng.random() < 0.3:
                _, n, u, v, w = rand_graph(rng, 60 * seed + 50 + rnd)
                srv.add_tenant(S.Tenant(f"a{rnd}", n, u, v, w, int(rng.integers(0, n))))
                graphs.append([u, v, w])
        for t in srv.admitted:
            ten = srv.tenants[t]
            p, d = srv.tree(t)
            u, v, w = graphs[t]
            check_against_oracle(ten.n, u, v, w, np.zeros(0, D.CHANGE_DTYPE), ten.src, p, d, f"server seed {seed} final {t}")
    return "ok"


POOL_CASES = int(os.environ.get("DSSSP_SOAK_POOL_CASES", "60"))


@pytest.mark.parametrize("block", range(3))
def test_random_pool_cases(block):
    per = (POOL_CASES + 2) // 3
    done = [pool_case(s) for s in range(block * per, min(POOL_CASES, (block + 1) * per))]
    assert "ok" in done


@pytest.mark.parametrize("block", range(3))
def test_random_server_cases(block):
    per = (POOL_CASES + 2) // 3
    done = [server_case(s) for s in range(block * per, min(POOL_CASES, (block + 1) * per))]
    assert "ok" in done
