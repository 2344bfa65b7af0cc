"""Failure detection without a GPU fault: a grid barrier of the update kernel whose wait runs
out (one CTA arrives late through a bounded test hook; the others give up after a small poll
limit) fails the batch with DSSSP_E_TIMEOUT, and the same graph then works again."""
import pytest

import dynamicssspv2_gb300 as D
from tests.common import check_against_oracle

pytestmark = pytest.mark.gpu


def test_barrier_timeout_is_reported_and_the_device_stays_usable():
    n, m = 20000, 80000
    u, v, w = D.gen_er(n, m, 1, 100, 61)
    ch = D.gen_changes(n, u, v, w, 2000, 2000, seed=62)
    with D.Graph(n, u, v, w) as g:
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
