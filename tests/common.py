"""Helpers shared by the tests: golden fixtures and engine-vs-oracle comparison."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

import dynamicssspv2_gb300 as D
from oracle import pyoracle as O

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden.json"


def golden_cases():
    return json.loads(GOLDEN.read_text())["cases"]


def case_arrays(case):
    e = np.array(case["edges"], np.int64).reshape(-1, 3)
    ch = np.array(case["changes"], np.int64).reshape(-1, 4)
    changes = D.make_changes(ch[:, 0], ch[:, 1], ch[:, 2], ch[:, 3]) if len(ch) else np.zeros(0, D.CHANGE_DTYPE)
    return e[:, 0].astype(np.int32), e[:, 1].astype(np.int32), e[:, 2].astype(np.int32), changes


def tree_from_rows(n, rows):
    """SSSP file rows (node, parent, dist) -> (parent, dist) as the engine loads them."""
    parent = np.full(n, -1, np.int32)
    dist = np.full(n, -1, np.int64)
    for node, p, d in rows:
        parent[node] = p
        dist[node] = d if p != -1 else -1
    return parent, dist


def check_against_oracle(n, u, v, w, changes, src, parent, dist, where=""):
    """Bit-exact distances against the oracle's Dijkstra on the updated graph, and a valid
    shortest-path tree (parents may differ on ties)."""
    g = O.updated_graph(n, u, v, w, changes)
    od, op = O.dijkstra(n, g, src)
    reach_e = parent != -1
    reach_o = op != -1
    bad = np.flatnonzero(reach_e != reach_o)
    assert len(bad) == 0, f"{where}: reachability differs at {bad[:10]}"
    diff = np.flatnonzero(dist != od)
    assert len(diff) == 0, f"{where}: {len(diff)} distances differ, e.g. v={diff[:5]} got {dist[diff[:5]]} want {od[diff[:5]]}"
    res = O.validate(n, g, src, dist, parent)
    assert res == 0, f"{where}: invalid tree: {res}"


def lines_after(n, u, v, w, changes):
    """The edge lines of the graph after a batch (the reference's semantics: insertions
    appended, then every line matching a deletion's pair and weight removed), for chaining
    batches in the oracle."""
    _, kept = O.updated_graph(n, u, v, w, changes, return_kept=True)
    ins = changes[changes["op"] == 1]
    lu = np.concatenate([u, ins["u"]]).astype(np.int32)
    lv = np.concatenate([v, ins["v"]]).astype(np.int32)
    lw = np.concatenate([w, ins["w"]]).astype(np.int32)
    keep = kept[: len(lu)].astype(bool)
    return lu[keep], lv[keep], lw[keep]
