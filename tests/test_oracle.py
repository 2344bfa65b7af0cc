"""The CPU oracle, pinned against the reference itself (golden fixtures made by running the
reference's compiled sources, tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.common import case_arrays, golden_cases

CASES = golden_cases()


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_dijkstra_matches_reference_seq(case):
    """orc_dijkstra on orc_updated_graph == seqSSSPwithDist_undir.cpp run on the updated graph
    file: distances and parents bit-exact (same 1000*N cap, same row order)."""
    n = case["n"]
    u, v, w, ch = case_arrays(case)
    g = O.updated_graph(n, u, v, w, ch)
    dist, parent = O.dijkstra(n, g, 0, inf_cap=1000 * n)
    assert parent.tolist() == case["seq_after"]["parent"]
    assert dist.tolist() == case["seq_after"]["dist"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_ref_update_restatement_matches_reference_kernels(case):
    """orc_ref_update == the reference's own kernels replayed thread by thread."""
    n = case["n"]
    u, v, w, ch = case_arrays(case)
    rows = np.array(case["sssp_in"], np.int64).reshape(-1, 3)
    ip, idist = O.read_sssp_semantics(n, rows[:, 0], rows[:, 1], rows[:, 2])
    d, p, rounds = O.ref_update(n, u, v, w, ch, ip, idist)
    assert d.tolist() == case["ref_update"]["dist"]
    assert p.tolist() == case["ref_update"]["parent"]
    assert rounds == (case["ref_update"]["rounds"]["rounds_del"], case["ref_update"]["rounds"]["rounds_relax"])


def test_reference_update_disagrees_with_recompute_only_on_mid():
    """The reference's CUDA update equals a recompute of the updated graph on every golden case
    but `mid`, where it seeds relaxation from an insertion that the same batch deletes again
    (gpuFunctions_undir.cuh:217-251 runs after the tombstoning of 201-213).  The GPU parity
    tests compare the engine with the reference update on all the others."""
    differ = []
    for c in CASES:
        ref = np.array(c["ref_update"]["dist"])
        sp = np.array(c["seq_after"]["parent"])
        sd = np.array(c["seq_after"]["dist"])
        unreach = ref >= 999999
        if not (np.array_equal(sp == -1, unreach) and np.array_equal(sd[~unreach], ref[~unreach])):
            differ.append(c["name"])
    assert differ == ["mid"]


def test_sample_known_answer():
    """README.md:18 sample: delete 0-1 (w2), insert 0-4 (w4) and 1-4 (w0)."""
    case = CASES[0]
    assert case["name"] == "sample"
    assert case["seq_after"]["dist"] == [0, 4, 6, 6, 4, 9]
    u, v, w, ch = case_arrays(case)
    g = O.updated_graph(6, u, v, w, ch)
    dist, parent = O.dijkstra(6, g, 0)
    assert dist.tolist() == [0, 4, 6, 6, 4, 9]
    assert parent[2] in (0, 4)  # tie: 0->2 = 6 and 0->4->2 = 6
    assert O.validate(6, g, 0, dist, parent) == 0


def test_updated_graph_semantics():
    # base: 0-1 w5 twice, 1-2 w3; insert 0-1 w5 and 0-2 w9; delete 1-0 w5 and 2-1 w4 (absent)
    u = np.array([0, 0, 1], np.int32)
    v = np.array([1, 1, 2], np.int32)
    w = np.array([5, 5, 3], np.int32)
    ch = np.zeros(4, [("u", "<i4"), ("v", "<i4"), ("w", "<i4"), ("op", "<i4")])
    ch[:] = [(0, 1, 5, 1), (0, 2, 9, 1), (1, 0, 5, 0), (2, 1, 4, 0)]
    g, kept = O.updated_graph(3, u, v, w, ch, return_kept=True)
    # every 0-1 w5 copy (two base + one inserted) is gone; 1-2 and 0-2 remain
    assert kept[:5].tolist() == [0, 0, 1, 0, 1]
    assert g.off.tolist() == [0, 1, 2, 4]
    rows = [list(zip(g.col[g.off[r]:g.off[r + 1]].tolist(), g.wt[g.off[r]:g.off[r + 1]].tolist())) for r in range(3)]
    assert rows == [[(2, 9)], [(2, 3)], [(1, 3), (0, 9)]]


def test_validator_rejects_planted_errors():
    u = np.array([0, 1, 2, 0], np.int32)
    v = np.array([1, 2, 3, 3], np.int32)
    w = np.array([1, 1, 1, 5], np.int32)
    g = O.csr(4, u, v, w)
    dist, parent = O.dijkstra(4, g, 0)
    assert dist.tolist() == [0, 1, 2, 3]
    assert O.validate(4, g, 0, dist, parent) == 0
    bad = dist.copy()
    bad[3] = 4  # not the shortest
    assert O.validate(4, g, 0, bad, parent) != 0
    badp = parent.copy()
    badp[3] = 0  # edge 0-3 has weight 5, not 3
    assert O.validate(4, g, 0, dist, badp) != 0
    # a zero-weight cycle: 1 <-> 2 with w 0 and equal distances
    u2 = np.array([0, 1, 0], np.int32)
    v2 = np.array([1, 2, 2], np.int32)
    w2 = np.array([3, 0, 3], np.int32)
    g2 = O.csr(3, u2, v2, w2)
    d2 = np.array([0, 3, 3], np.int64)
    assert O.validate(3, g2, 0, d2, np.array([0, 0, 0], np.int32)) == 0
    assert O.validate(3, g2, 0, d2, np.array([0, 2, 1], np.int32)) != 0  # cycle
    unreach = np.array([0, 3, -1], np.int64)
    assert O.validate(3, g2, 0, unreach, np.array([0, 0, -1], np.int32)) != 0  # 2 is reachable


def test_dijkstra_exact_mode_ignores_cap():
    # a path whose length exceeds 1000*N: the reference's cap calls it unreachable
    u = np.array([0, 1], np.int32)
    v = np.array([1, 2], np.int32)
    w = np.array([600000, 600000], np.int32)
    g = O.csr(3, u, v, w)
    d_cap, p_cap = O.dijkstra(3, g, 0, inf_cap=3000)
    assert p_cap.tolist() == [0, -1, -1]
    d, p = O.dijkstra(3, g, 0)
    assert d.tolist() == [0, 600000, 1200000] and p.tolist() == [0, 0, 1]


def test_reference_dijkstra_timing_harness():
    """oracle/time_ref.py times the reference's compiled djk (oracle/_ref/ref_time) and the
    restatement on the same updated graph (here the small ER workload)."""
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    if not (root / "oracle" / "_ref" / "ref_time").exists():
        pytest.skip("the reference's sources were not available to build oracle/_ref/ref_time")
    out = subprocess.run([sys.executable, str(root / "oracle" / "time_ref.py"), "--workload", "er10k", "--reps", "1"],
                         capture_output=True, text=True, timeout=300, check=True).stdout
    assert "reference djk" in out and "oracle restatement" in out


def test_oracle_generators_match_the_library():
    """The oracle's restatement of the seeded generators (used by bench.py's CPU reference arm,
    which loads no product library) gives exactly the library's edge lists, change batches and
    highest-degree vertex."""
    import dynamicssspv2_gb300 as D

    for n, m, wlo, whi, seed in ((1000, 4000, 1, 100, 5), (5000, 30000, 1, 60, 7)):
        a, b = D.gen_er(n, m, wlo, whi, seed), O.gen_er(n, m, wlo, whi, seed)
        assert all(np.array_equal(x, y) for x, y in zip(a, b))
        c1 = D.gen_changes(n, *a, 300, 300, seed=3, wlo=2, whi=9)
        c2 = O.gen_changes(n, *b, 300, 300, 0, 0, 0.0, 0.0, 0.0, 2, 9, 3)
        assert np.array_equal(c1.view(np.int32), c2.view(np.int32))
    for scale, m in ((10, 3000), (14, 100000)):
        n = 1 << scale
        a = D.gen_rmat(scale, m, 0.57, 0.19, 0.19, 1, 100, seed=0)
        b = O.gen_rmat(scale, m, 0.57, 0.19, 0.19, 1, 100, 0)
        assert all(np.array_equal(x, y) for x, y in zip(a, b))
        assert D.max_degree_vertex(n, a[0], a[1]) == O.max_degree_vertex(n, b[0], b[1])
        c1 = D.gen_changes(n, *a, 500, 400, D.INS_RMAT, scale, 0.57, 0.19, 0.19, 1, 100, seed=1)
        c2 = O.gen_changes(n, *b, 500, 400, 1, scale, 0.57, 0.19, 0.19, 1, 100, 1)
        assert np.array_equal(c1.view(np.int32), c2.view(np.int32))
