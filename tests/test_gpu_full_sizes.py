"""Parity at the full sizes of the plain configurations (ER-10k, RMAT-22 with a 10^6-change
batch, the 4096x4096 grid with 10^5 changes): the device certificate of the tree before and
after the batch, and the distances after it bit-exact against the oracle's Dijkstra on the
updated graph, parents a valid shortest-path tree."""
import numpy as np
import pytest

import bench
import dynamicssspv2_gb300 as D
from tests.common import check_against_oracle

pytestmark = pytest.mark.gpu

OPTS = {"er10k": {}, "rmat22": {}, "grid4096": {"delta": 3000}}


@pytest.mark.parametrize("workload", sorted(OPTS))
def test_full_size_batch_is_exact(workload):
    n, u, v, w, src, ch = bench.make_inputs(workload)
    with D.Graph(n, u, v, w, **OPTS[workload]) as g:
        g.tree_compute(src)
        c0 = g.validate()
        assert c0["violations"] == 0 and c0["roots"] == 1
        st = g.apply_batch(ch)
        c1 = g.validate()
        assert c1["violations"] == 0 and c1["roots"] == 1, c1
        p, d = g.tree_read()
    assert st.n_ins + st.n_del == len(ch) and st.n_invalidated > 0
    assert d[src] == 0 and p[src] == src
    check_against_oracle(n, u, v, w, ch, src, p, d, workload)
    assert np.count_nonzero(p >= 0) > n // 4
