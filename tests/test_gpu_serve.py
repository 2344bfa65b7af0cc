"""Serving layer on the GPU: continuous batching must give every request the result it gets
alone (distances bit-exact, parents a valid tree of the tenant's graph after that request);
tenants are admitted by memory footprint."""
import numpy as np
import pytest

import dynamicssspv2_gb300 as D
from dynamicssspv2_gb300.serve import Request, Server, Tenant, estimate_footprint, random_batch, summarize
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def make_tenants(count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(300, 4000))
        m = n * int(rng.integers(2, 5))
        u, v, w = D.gen_er(n, m, 1, 100, seed * 100 + i)
        out.append(Tenant(f"t{i}", n, u, v, w, src=int(rng.integers(0, n))))
    return out


def apply_lines(n, u, v, w, ch):
    _, kept = O.updated_graph(n, u, v, w, ch, return_kept=True)
    ins = ch[ch["op"] == 1]
    lu = np.concatenate([u, ins["u"]]).astype(np.int32)
    lv = np.concatenate([v, ins["v"]]).astype(np.int32)
    lw = np.concatenate([w, ins["w"]]).astype(np.int32)
    keep = kept[: len(lu)].astype(bool)
    return lu[keep], lv[keep], lw[keep]


def test_each_result_same_alone_and_in_the_mix():
    tenants = make_tenants(6, 1)
    rng = np.random.default_rng(2)
    reqs = []
    for t, ten in enumerate(tenants):
        for j in range(4):
            reqs.append(Request(t, float(rng.uniform(0, 0.03)), random_batch(rng, ten, int(rng.integers(10, 300)))))
    # all requests at once: every epoch mixes several tenants; a tiny tombstone threshold makes
    # the server compact once it is idle
    with Server(tenants, compact_dead_frac=1e-4) as srv:
        out = srv.serve(reqs, record=True, realtime=False)
        assert srv.validate() == {"violations": 0, "roots": len(tenants)}
    assert srv.compactions > 0
    epochs = {}
    for r in out:
        epochs.setdefault(r.epoch, []).append(r)
    assert max(len(e) for e in epochs.values()) > 1, "no epoch mixed several tenants"
    for t, ten in enumerate(tenants):
        mine = sorted([r for r in out if r.tenant == t], key=lambda r: r.arrival)
        assert [r.epoch for r in mine] == sorted(r.epoch for r in mine)  # arrival order kept
        u, v, w = ten.u, ten.v, ten.w
        with D.Graph(ten.n, u, v, w) as g:  # alone: the same batches one by one
            g.tree_compute(ten.src)
            for r in mine:
                g.apply_batch(r.changes)
                p_alone, d_alone = g.tree_read()
                p_mix, d_mix = r.result
                assert np.array_equal(d_mix, d_alone), f"tenant {t} request {r.rid}: mix differs from alone"
                u, v, w = apply_lines(ten.n, u, v, w, r.changes)
                gr = O.csr(ten.n, u, v, w)
                od, op = O.dijkstra(ten.n, gr, ten.src)
                assert np.array_equal(d_mix, od)
                assert O.validate(ten.n, gr, ten.src, d_mix, p_mix) == 0


def test_admission_by_footprint_and_refusal():
    tenants = make_tenants(4, 3)
    fp = [estimate_footprint(t.n, len(t.u)) for t in tenants]
    budget = fp[0] + fp[1] + fp[2] // 2
    rng = np.random.default_rng(4)
    reqs = [Request(t, 0.0, random_batch(rng, tenants[t], 50)) for t in range(4)]
    expect, used = [], 0
    for i, f in enumerate(fp):  # admitted in order while the footprint fits
        if used + f <= budget:
            expect.append(i)
            used += f
    with Server(tenants, memory_budget=budget) as srv:
        assert srv.admitted == expect and 2 not in expect
        out = srv.serve(reqs)
    refused = {r.tenant for r in out if r.refused}
    assert 2 in refused and all(r.refused == (r.tenant not in srv.admitted) for r in out)
    s = summarize(out)
    assert s["refused"] == len(refused) and s["served"] == 4 - len(refused)


def test_saturated_serving_batches_all_tenants():
    tenants = make_tenants(5, 5)
    rng = np.random.default_rng(6)
    reqs = [Request(t, 0.0, random_batch(rng, tenants[t], 100)) for t in range(5) for _ in range(3)]
    with Server(tenants) as srv:
        out = srv.serve(reqs, realtime=False)
    assert srv.epochs == 3  # every epoch takes one request of each tenant
    assert summarize(out)["mean_requests_per_epoch"] == 5


def test_malformed_requests_fail_alone():
    """Requests naming a vertex outside their tenant's graph or inserting a negative weight fail
    on arrival; the requests around them are served exactly as if they were not there."""
    tenants = make_tenants(3, 7)
    rng = np.random.default_rng(8)
    good = [Request(t, 0.001 * i, random_batch(rng, tenants[t], 80)) for i, t in enumerate([0, 1, 2, 0, 1, 2])]
    bad_vertex = random_batch(rng, tenants[1], 20)
    bad_vertex["v"][3] = tenants[1].n + 7
    bad_weight = random_batch(rng, tenants[2], 20)
    bad_weight["w"][bad_weight["op"] == 1] = -5
    reqs = good + [Request(1, 0.0025, bad_vertex), Request(2, 0.0035, bad_weight)]
    with Server(tenants) as srv:
        out = srv.serve(reqs, record=True)
    failed = [r for r in out if r.error is not None]
    assert len(failed) == 2 and all(r.result is None for r in failed)
    assert "vertex" in failed[0].error and "negative" in failed[1].error
    s = summarize(out)
    assert s["failed"] == 2 and s["served"] == len(good)
    for t, ten in enumerate(tenants):
        mine = sorted([r for r in out if r.tenant == t and r.error is None], key=lambda r: r.arrival)
        with D.Graph(ten.n, ten.u, ten.v, ten.w) as g:
            g.tree_compute(ten.src)
            for r in mine:
                g.apply_batch(r.changes)
                assert np.array_equal(g.tree_read()[1], r.result[1])


def test_failed_epoch_is_recovered_and_serving_stays_exact():
    """The first epoch's update kernel times out (bounded test hooks on the pool's graph); the
    server recovers it by recomputing every tenant's tree on the device, serves its requests
    with `recomputed` set, and every later request is exact: each tenant equals the oracle on
    its edge lists after all requests, and the certificate holds."""
    tenants = make_tenants(5, 11)
    rng = np.random.default_rng(12)
    first = [Request(t, 0.0, random_batch(rng, tenants[t], 150)) for t in range(5)]
    later = [Request(t, 0.0, random_batch(rng, tenants[t], 150)) for t in range(5) for _ in range(2)]
    with Server(tenants) as srv:
        srv.debug_set(D.DEBUG_SPIN_LIMIT, 4096)
        srv.debug_set(D.DEBUG_STALL_US, 200_000)  # one launch: the first epoch's
        out1 = srv.serve(first, realtime=False)
        assert all(r.recomputed and r.error is None for r in out1), [(r.recomputed, r.error) for r in out1]
        assert srv.recovered_epochs == 1
        srv.debug_set(D.DEBUG_SPIN_LIMIT, 0)
        out2 = srv.serve(later, realtime=False)
        assert all(not r.recomputed and r.error is None and not r.refused for r in out2)
        assert srv.validate() == {"violations": 0, "roots": len(tenants)}
        for t, ten in enumerate(tenants):
            u, v, w = ten.u, ten.v, ten.w
            for r in sorted([r for r in out1 + out2 if r.tenant == t], key=lambda r: (r.epoch, r.arrival)):
                u, v, w = apply_lines(ten.n, u, v, w, r.changes)
            gr = O.csr(ten.n, u, v, w)
            od, _ = O.dijkstra(ten.n, gr, ten.src)
            p, d = srv.tree(t)
            assert np.array_equal(d, od), f"tenant {t}"
            assert O.validate(ten.n, gr, ten.src, d, p) == 0


def test_tenants_join_and_leave_while_serving():
    """Admission follows the budget as tenants come and go: a tenant that does not fit waits
    (its requests are refused), and is admitted -- its tree built on the device -- when a
    removal frees memory; a tenant added at run time is admitted into free ids; a removed
    tenant's later requests are refused.  Every served request's result equals its tenant's
    batches applied alone, and the oracle's tree."""
    sizes = [2000, 12000, 1500, 3000, 2500]
    ten = []
    for i, n in enumerate(sizes):
        u, v, w = D.gen_er(n, 3 * n, 1, 100, 500 + i)
        ten.append(Tenant(f"t{i}", n, u, v, w, src=i))
    tenants, extra = ten[:4], ten[4]
    fp = [estimate_footprint(t.n, len(t.u)) for t in ten]
    budget = fp[0] + fp[1] + fp[2] + fp[3] // 4  # tenant 3 waits; removing tenant 1 makes room
    assert fp[1] > fp[3] + fp[4]
    rng = np.random.default_rng(22)
    phase1, phase2 = [], []
    with Server(tenants, memory_budget=budget, reserve_vertices=extra.n) as srv:
        assert srv.admitted == [0, 1, 2] and srv.state(3) == D.TENANT_WAITING
        phase1 = srv.serve([Request(t, 0.0, random_batch(rng, tenants[t], 60)) for t in range(4)], record=True)
        assert {r.tenant for r in phase1 if r.refused} == {3}
        srv.remove_tenant(1)  # frees memory and ids: tenant 3 comes in
        assert srv.state(1) == D.TENANT_REMOVED and srv.state(3) == D.TENANT_ADMITTED
        t4 = srv.add_tenant(extra)
        assert t4 == 4 and srv.state(4) == D.TENANT_ADMITTED
        assert srv.admitted == [0, 2, 3, 4]
        phase2 = srv.serve([Request(t, 0.0, random_batch(rng, srv.tenants[t], 60)) for t in range(5)
                            for _ in range(2)], record=True, realtime=False)
        assert {r.tenant for r in phase2 if r.refused} == {1}
        assert all(r.error is None for r in phase1 + phase2)
        assert srv.validate() == {"violations": 0, "roots": 4}
    for t in (0, 1, 2, 3, 4):
        reqs = sorted([r for r in phase1 + phase2 if r.tenant == t and not r.refused],
                      key=lambda r: (r.epoch, r.arrival))
        tn = ten[t]
        with D.Graph(tn.n, tn.u, tn.v, tn.w) as g:  # alone
            g.tree_compute(tn.src)
            u, v, w = tn.u, tn.v, tn.w
            for r in reqs:
                g.apply_batch(r.changes)
                assert np.array_equal(g.tree_read()[1], r.result[1]), f"tenant {t}: mix differs from alone"
                u, v, w = apply_lines(tn.n, u, v, w, r.changes)
            if reqs:
                gr = O.csr(tn.n, u, v, w)
                od, _ = O.dijkstra(tn.n, gr, tn.src)
                assert np.array_equal(reqs[-1].result[1], od)
                assert O.validate(tn.n, gr, tn.src, reqs[-1].result[1], reqs[-1].result[0]) == 0


def test_pool_graphs_added_and_removed():
    """A pool with a vertex reserve: a graph added later gets the tree a graph store of its own
    computes, without changing the others; a removed graph's ids are reused by a later one;
    a range with edges to the rest of the store cannot be cleared."""
    from dynamicssspv2_gb300.pool import GraphPool

    base = [(n, *D.gen_er(n, 3 * n, 1, 100, 600 + i)) for i, n in enumerate((700, 1300))]
    late = [(n, *D.gen_er(n, 3 * n, 1, 100, 700 + i)) for i, n in enumerate((900, 1100, 600))]
    with GraphPool(base, reserve_vertices=2000) as pool:
        pool.tree_compute([0, 0])
        before = pool.tree_read()
        a = pool.add_graph(*late[0], src=3)
        assert pool.graph_range(a) == (2000, 900)
        for i in range(2):
            assert np.array_equal(pool.tree_read(i)[1], before[i][1])
        pool.remove_graph(0)
        b = pool.add_graph(*late[1], src=5)
        assert pool.graph_range(b) == (2900, 1100)  # the freed ids [0, 700) are too few
        c = pool.add_graph(*late[2], src=7)
        assert pool.graph_range(c) == (0, 600)  # reuses the removed graph's ids
        with pytest.raises(D.DsssspError) as e:
            pool.add_graph(*late[0], src=0)  # no free range of 900 ids is left
        assert e.value.code == D.E_OOM
        cert = pool.graph.validate()
        assert cert["violations"] == 0 and cert["roots"] == 4
        for gi, (n, u, v, w), src in ((a, late[0], 3), (b, late[1], 5), (c, late[2], 7), (1, base[1], 0)):
            with D.Graph(n, u, v, w) as g:
                g.tree_compute(src)
                assert np.array_equal(pool.tree_read(gi)[1], g.tree_read()[1]), f"graph {gi}"
        with pytest.raises(D.DsssspError) as e:
            pool.graph.clear_range(1000, 500)  # would cut graph 1 in two
        assert e.value.code == D.E_INVAL


def test_server_takes_options_from_the_tune_cache(tmp_path):
    """With tune_cache the server sets, per epoch, the cached options of the epoch's size class:
    a cache naming small_deg 8 and solo_waves 0 for every batch-size class of this pool is taken
    (the pool's graph carries them after serving) and the results stay exact."""
    import ctypes as C

    from dynamicssspv2_gb300.autotune import size_class

    tenants = make_tenants(4, 41)
    n = sum(t.n for t in tenants)
    entries = 2 * sum(len(t.u) for t in tenants)
    cache = tmp_path / "tune.txt"
    cache.write_text("".join(f"{size_class(n, entries, 1 << b)} 1.0 small_deg=8 solo_waves=0\n" for b in range(0, 14)))
    rng = np.random.default_rng(42)
    reqs = [Request(t, 0.0, random_batch(rng, tenants[t], 120)) for t in range(4) for _ in range(2)]
    with Server(tenants, tune_cache=str(cache)) as srv:
        out = srv.serve(reqs, record=True, realtime=False)
        g = D.Graph.__new__(D.Graph)  # the pool's graph, owned by the server (not closed here)
        g._h = C.c_void_p(D._lib.dsssp_pool_graph(D._lib.dsssp_server_pool(srv._h)))
        o = g.get_opts()
        g._h = C.c_void_p()
        assert o.small_deg == 8 and o.solo_waves == 0
    for t, ten in enumerate(tenants):
        with D.Graph(ten.n, ten.u, ten.v, ten.w) as g:
            g.tree_compute(ten.src)
            for r in sorted([r for r in out if r.tenant == t], key=lambda r: (r.epoch, r.arrival)):
                g.apply_batch(r.changes)
                assert np.array_equal(g.tree_read()[1], r.result[1])
