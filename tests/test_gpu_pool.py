"""Batching layer on the GPU: many graphs in one pooled graph store updated by one launch
sequence must give, per graph, exactly what the plain single-graph update gives; plus
multi-source trees, runtime option changes and the autotuner."""
import numpy as np
import pytest

import dynamicssspv2_gb300 as D
from dynamicssspv2_gb300.autotune import Autotuner
from dynamicssspv2_gb300.pool import GraphPool
from oracle import pyoracle as O
from tests.common import check_against_oracle

pytestmark = pytest.mark.gpu


def make_graphs(count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(10 ** rng.uniform(1.5, 4))
        m = min(n * int(rng.integers(1, 6)), n * (n - 1) // 2)
        u, v, w = D.gen_er(n, m, 1, 60, seed * 100 + i)
        k = max(2, int(m * rng.uniform(0.01, 0.2)))
        ch = D.gen_changes(n, u, v, w, k // 2, k - k // 2, seed=seed * 1000 + i)
        out.append((n, u, v, w, ch))
    return out


def test_pool_equals_plain_per_graph():
    graphs = make_graphs(12, 1)
    with GraphPool([(n, u, v, w) for n, u, v, w, _ in graphs]) as pool:
        pool.tree_compute([0] * len(graphs))
        st = pool.apply([(i, g[4]) for i, g in enumerate(graphs)])
        assert st.n_ins + st.n_del == sum(len(g[4]) for g in graphs)
        trees = pool.tree_read()
    for i, ((n, u, v, w, ch), (p, d)) in enumerate(zip(graphs, trees)):
        check_against_oracle(n, u, v, w, ch, 0, p, d, f"pooled graph {i}")
        with D.Graph(n, u, v, w) as g:
            g.tree_compute(0)
            g.apply_batch(ch)
            p1, d1 = g.tree_read()
        assert np.array_equal(d, d1), f"graph {i}: pooled and plain distances differ"


def test_pool_partial_batches_and_forest_load():
    graphs = make_graphs(6, 2)
    trees = []
    for n, u, v, w, _ in graphs:
        d, p = O.dijkstra(n, O.csr(n, u, v, w), 0)
        trees.append((p, d))
    with GraphPool([(n, u, v, w) for n, u, v, w, _ in graphs]) as pool:
        pool.forest_load(trees)
        chosen = [1, 3, 4]
        pool.apply([(i, graphs[i][4]) for i in chosen])
        out = pool.tree_read()
        for i, (n, u, v, w, ch) in enumerate(graphs):
            p, d = out[i]
            if i in chosen:
                check_against_oracle(n, u, v, w, ch, 0, p, d, f"graph {i}")
            else:
                assert np.array_equal(d, trees[i][1]) and np.array_equal(p, trees[i][0])
        with pytest.raises(D.DsssspError):  # two batches of one graph in one union
            pool.apply([(1, graphs[1][4]), (1, graphs[1][4])])
        bad = graphs[2][4].copy()
        bad["u"][0] = graphs[2][0]  # one past the graph's last vertex
        with pytest.raises(D.DsssspError) as e:
            pool.apply([(2, bad)])
        assert e.value.code == D.E_BAD_VERTEX and "graph 2" in str(e.value)


def test_multi_source_distances():
    n, m = 3000, 12000
    u, v, w = D.gen_er(n, m, 1, 100, 5)
    srcs = [0, 1234, 2999]
    g = O.csr(n, u, v, w)
    best = np.full(n, np.iinfo(np.int64).max)
    for s in srcs:
        d, p = O.dijkstra(n, g, s)
        best = np.where((p != -1) & (d < best), d, best)
    with D.Graph(n, u, v, w) as G:
        G.tree_compute_multi(srcs)
        p, d = G.tree_read()
    reach = best != np.iinfo(np.int64).max
    assert np.array_equal(p != -1, reach)
    assert np.array_equal(d[reach], best[reach])
    assert all(p[s] == s and d[s] == 0 for s in srcs)


def test_set_opts_keeps_results_exact():
    n, m = 5000, 20000
    u, v, w = D.gen_er(n, m, 1, 100, 9)
    ch = D.gen_changes(n, u, v, w, 500, 500, seed=10)
    with D.Graph(n, u, v, w) as g:
        g.tree_compute(0)
        g.snapshot()
        for over in ({"small_deg": 8}, {"large_deg": 16, "chunk": 64}, {"bfs_levels": 0}, {"block": 128}):
            o = g.get_opts()
            for k, val in over.items():
                setattr(o, k, val)
            g.set_opts(o)
            g.restore()
            g.apply_batch(ch)
            p, d = g.tree_read()
            check_against_oracle(n, u, v, w, ch, 0, p, d, str(over))
        bad = g.get_opts()
        bad.small_deg = 6
        with pytest.raises(D.DsssspError):
            g.set_opts(bad)


def test_autotuner_picks_and_caches(tmp_path):
    graphs = make_graphs(8, 3)
    cache = tmp_path / "tune.txt"
    with GraphPool([(n, u, v, w) for n, u, v, w, _ in graphs]) as pool:
        pool.tree_compute([0] * len(graphs))
        before = pool.graph.tree_read()
        union = pool.union_batch([(i, g[4]) for i, g in enumerate(graphs)])
        res = Autotuner(cache, reps=1).tune(pool.graph, union)
        assert not res["cached"] and res["trials"] >= 4 and cache.exists()
        after = pool.graph.tree_read()
        assert np.array_equal(before[1], after[1])  # tuning leaves the distances as they were
        res2 = Autotuner(cache).tune(pool.graph, union)
        assert res2["cached"] and res2["opts"] == res["opts"]
        pool.graph.apply_batch(union)
        for i, (p, d) in enumerate(pool.tree_read()):
            n, u, v, w, ch = graphs[i]
            check_against_oracle(n, u, v, w, ch, 0, p, d, f"tuned graph {i}")
