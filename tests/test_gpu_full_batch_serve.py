"""The batching and serving workloads at their full sizes on the GPU, checked against the oracle.

batch256: 256 Erdos-Renyi graphs (n log-uniform in [1e3, 1e6], average degree 8), each with its
own batch of 0.1-10 % of its edges, applied as one union batch by one launch sequence of a
pooled store.  The device certificate covers every graph's tree before and after the batch
(one root per graph, no violation); eight graphs -- the smallest, the largest and six drawn at
random -- are compared bit-exact with the oracle's Dijkstra on their updated graphs.  Run with
the default options and with the walk switched to pointer jumping at once (bfs_levels 0, the
setting the autotuner picks for this workload).

serve: the resident RMAT scale-24 graph (134,217,728 edges) and 32 Erdos-Renyi tenants of
1e5-2e6 vertices in one server; warm-up requests, then a Poisson stream.  Every request must be
served, the certificate must hold for every tenant, and four tenants -- the two smallest, one
of middle size and the largest Erdos-Renyi tenant -- must equal the oracle's Dijkstra on their
edge lists after all requests (the reference's batch semantics, applied on the host).
"""
import numpy as np
import pytest

import bench
import dynamicssspv2_gb300 as D
from dynamicssspv2_gb300.pool import GraphPool
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch256_inputs():
    return bench.make_batch_inputs("batch256")


@pytest.mark.parametrize("opts", [{}, {"bfs_levels": 0}], ids=["default", "pointer_jumping"])
def test_batch256_full_size_exact(batch256_inputs, opts):
    items = batch256_inputs
    wl = bench.WORKLOADS["batch256"]
    assert len(items) == wl["count"]
    with GraphPool([(n, u, v, w) for n, u, v, w, _ in items], slack_pct=wl["slack_pct"],
                   slack_min=wl["slack_min"], **opts) as pool:
        pool.tree_compute([0] * len(items))
        before = pool.graph.validate()
        assert before["violations"] == 0 and before["roots"] == len(items), before
        st = pool.apply([(i, it[4]) for i, it in enumerate(items)])
        assert st.n_ins + st.n_del == sum(len(it[4]) for it in items)
        after = pool.graph.validate()
        assert after["violations"] == 0 and after["roots"] == len(items), after
        sizes = np.array([it[0] for it in items])
        rng = np.random.default_rng(7)
        sample = {int(np.argmin(sizes)), int(np.argmax(sizes))}
        while len(sample) < 8:
            sample.add(int(rng.integers(0, len(items))))
        for i in sorted(sample):
            n, u, v, w, ch = items[i]
            p, d = pool.tree_read(i)
            g = O.updated_graph(n, u, v, w, ch)
            od, op = O.dijkstra(n, g, 0)
            assert np.array_equal(d, od), f"graph {i} (n={n}): {int((d != od).sum())} distances differ"
            assert np.array_equal(p == -1, op == -1), f"graph {i}: reachability differs"
            assert O.validate(n, g, 0, d, p) == 0, f"graph {i}: invalid tree"


def test_serve_full_size_exact():
    from dynamicssspv2_gb300.serve import Server, summarize

    wl = bench.WORKLOADS["serve"]
    tenants = bench.make_serve_tenants("serve")
    assert len(tenants) == wl["tenants"] + 1 and tenants[0].n == 1 << wl["rmat_scale"]
    assert len(tenants[0].u) == wl["rmat_m"]
    ers = sorted(range(1, len(tenants)), key=lambda t: tenants[t].n)
    checked = [ers[0], ers[1], ers[len(ers) // 2], ers[-1]]
    tracker = bench.EdgeTracker(tenants, checked)
    with Server(tenants, slack_pct=50, slack_min=16) as srv:
        assert len(srv.admitted) == len(tenants)
        warm = bench.serve_requests("serve", tenants, 2 * len(tenants), 0, 1)
        srv.serve(warm, realtime=False)
        tracker.track(warm)
        stream = bench.serve_requests("serve", tenants, 300, 3000.0, 5)
        srv.serve(stream)
        tracker.track(stream)
        s = summarize(stream)
        assert s["served"] == len(stream) and s["failed"] == 0 and s["refused"] == 0, s
        cert = srv.validate()
        assert cert == {"violations": 0, "roots": len(tenants)}, cert
        for t in checked:
            p, d = srv.tree(t)
            n = tenants[t].n
            g = O.csr(n, *tracker.lines[t])
            od, op = O.dijkstra(n, g, tenants[t].src)
            assert np.array_equal(d, od), f"tenant {t} (n={n}): {int((d != od).sum())} distances differ"
            assert np.array_equal(p == -1, op == -1), f"tenant {t}: reachability differs"
            assert O.validate(n, g, tenants[t].src, d, p) == 0, f"tenant {t}: invalid tree"
