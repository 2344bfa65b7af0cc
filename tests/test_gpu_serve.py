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
