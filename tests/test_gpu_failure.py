"""Failure detection without a GPU fault: a grid barrier of the update kernel whose wait runs
out (one CTA arrives late through a bounded test hook; the others give up after a small poll
limit) fails the batch with DSSSP_E_TIMEOUT, and the same graph then works again.  With
recovery on (the default) the failed batch is finished by recomputing the tree from its root on
the updated graph: DSSSP_W_RECOMPUTED, and the result is exact."""
import numpy as np
import pytest

import dynamicssspv2_gb300 as D
from oracle import pyoracle as O
from tests.common import check_against_oracle, lines_after

pytestmark = pytest.mark.gpu


def test_barrier_timeout_is_reported_and_the_device_stays_usable():
    n, m = 20000, 80000
    u, v, w = D.gen_er(n, m, 1, 100, 61)
    ch = D.gen_changes(n, u, v, w, 2000, 2000, seed=62)
    with D.Graph(n, u, v, w, recover=0) as g:
        g.tree_compute(0)
        g.snapshot()
        g.debug_set(D.DEBUG_SPIN_LIMIT, 4096)  # a few ms of polling
        g.debug_set(D.DEBUG_STALL_US, 200_000)  # the last CTA arrives 200 ms late
        with pytest.raises(D.DsssspError) as e:
            g.apply_batch(ch)
        assert e.value.code == D.E_TIMEOUT
        g.debug_set(D.DEBUG_SPIN_LIMIT, 0)
        g.debug_set(D.DEBUG_STALL_US, 0)
        # the front kernels had applied the batch to the adjacency before the update kernel
        # gave up: go back to the snapshot and apply it again on the same graph and context
        g.restore()
        g.apply_batch(ch)
        p, d = g.tree_read()
        check_against_oracle(n, u, v, w, ch, 0, p, d, "after a timed-out batch")
        assert g.validate()["violations"] == 0


def test_timed_out_batch_is_recovered_exactly():
    """The same timed-out batch with recovery on: the call succeeds with DSSSP_W_RECOMPUTED
    (stats name the timeout), the tree is the oracle's for the updated graph, and the next
    batch on the same graph is exact too (the stall hook applied to one launch only)."""
    n, m = 20000, 80000
    u, v, w = D.gen_er(n, m, 1, 100, 61)
    ch = D.gen_changes(n, u, v, w, 2000, 2000, seed=62)
    with D.Graph(n, u, v, w) as g:
        g.tree_compute(0)
        g.debug_set(D.DEBUG_SPIN_LIMIT, 4096)
        g.debug_set(D.DEBUG_STALL_US, 200_000)
        st = g.apply_batch(ch)
        assert st.recovered_from == D.E_TIMEOUT and st.t_recompute_ms > 0
        p, d = g.tree_read()
        check_against_oracle(n, u, v, w, ch, 0, p, d, "recovered batch")
        assert g.validate() == {"violations": 0, "roots": 1, "first_bad": -1}
        g.debug_set(D.DEBUG_SPIN_LIMIT, 0)
        ch2 = D.gen_changes(n, u, v, w, 500, 500, seed=63)
        st2 = g.apply_batch(ch2)
        assert st2.recovered_from == 0
        assert g.validate()["violations"] == 0
        u1, v1, w1 = lines_after(n, u, v, w, ch)
        od, _ = O.dijkstra(n, O.updated_graph(n, u1, v1, w1, ch2), 0)
        assert np.array_equal(g.tree_read()[1], od)


def test_round_cap_is_recovered_exactly():
    """A round cap of 1 stops the update kernel with DSSSP_E_NO_CONVERGENCE after the batch's
    edits; recovery recomputes with the default cap and gives the exact tree."""
    n, m = 5000, 20000
    u, v, w = D.gen_er(n, m, 1, 100, 71)
    ch = D.gen_changes(n, u, v, w, 800, 800, seed=72)
    for recover in (1, 0):
        with D.Graph(n, u, v, w, recover=recover) as g:
            g.tree_compute(0)
            o = g.get_opts()
            o.max_rounds = 1
            g.set_opts(o)
            if recover:
                st = g.apply_batch(ch)
                assert st.recovered_from == D.E_NO_CONVERGENCE
                p, d = g.tree_read()
                check_against_oracle(n, u, v, w, ch, 0, p, d, "round cap")
            else:
                with pytest.raises(D.DsssspError) as e:
                    g.apply_batch(ch)
                assert e.value.code == D.E_NO_CONVERGENCE


def test_debug_hooks_reject_bad_values():
    u, v, w = D.gen_er(100, 300, seed=1)
    with D.Graph(100, u, v, w) as g:
        for what, value in ((D.DEBUG_SPIN_LIMIT, -1), (D.DEBUG_STALL_US, 2_000_000), (99, 1)):
            with pytest.raises(D.DsssspError) as e:
                g.debug_set(what, value)
            assert e.value.code == D.E_INVAL


def test_invalid_options_are_refused():
    u, v, w = D.gen_er(100, 300, seed=1)
    for bad in ({"timing": 3}, {"timing": -1}, {"small_deg": 6}, {"block": 512}, {"delta": -2}):
        with pytest.raises(D.DsssspError) as e:
            D.Graph(100, u, v, w, **bad)
        assert e.value.code == D.E_INVAL, bad
    with D.Graph(100, u, v, w) as g:
        o = g.get_opts()
        o.timing = 7
        with pytest.raises(D.DsssspError) as e:
            g.set_opts(o)
        assert e.value.code == D.E_INVAL
