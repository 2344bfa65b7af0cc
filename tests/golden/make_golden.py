"""Generates tests/golden/golden.json by running the reference itself.

Runs only where the reference sources are present (it builds oracle/_ref/ first):
  - oracle/_ref/op_ssspSeq  = seqSSSPwithDist_undir.cpp compiled as-is (initial trees and the
                              recomputed tree of the updated graph);
  - oracle/_ref/ref_update  = the reference's readers and update kernels replayed on the CPU
                              (oracle/ref_harness.cpp).
Case 0 is the reference's own sample (graph.txt / SSSP.txt / cE.txt, README.md:18).  The
other cases are seeded random graphs with the edge cases the engine must handle: weight-0
edges, parallel edges, deletions of absent edges, insert+delete of the same edge in one batch,
disconnected vertices; and shaped ones: a cut-off subtree deeper than the walk's level limit,
a hub losing many edges, a source losing all of its edges, a batch of ignored records only,
repeated records, a grid with cuts and shortcuts, skewed endpoints (hubs), a cut-off subtree
reattached by an insertion of the same batch, weights of 0 and 1 only.  The updated-graph file given to op_ssspSeq is built here in plain
Python from the batch semantics (insertions appended, then every line matching a deletion's
endpoint pair and weight removed), independently of oracle/oracle.c.

usage: DSSSP_REFERENCE=<reference source dir> python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
REF = Path(os.environ.get("DSSSP_REFERENCE", ""))
REFBIN = ROOT / "oracle" / "_ref"


def build_ref() -> None:
    """oracle/_ref/ from the reference's sources in DSSSP_REFERENCE."""
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "all", "ref", f"REF={REF}"], check=True)


def write_lines(path: Path, rows) -> None:
    path.write_text("".join(" ".join(str(x) for x in r) + "\n" for r in rows))


def run_seq(graph: Path, n: int):
    out = subprocess.run([str(REFBIN / "op_ssspSeq"), str(graph), str(n)], check=True, capture_output=True,
                         text=True).stdout
    parent = [0] * n
    dist = [0.0] * n
    for line in out.splitlines():
        f = line.split()
        if len(f) < 3:
            continue
        i = int(f[0])
        parent[i] = int(f[1])
        dist[i] = float(f[2])
    return parent, dist


def run_ref_update(graph: Path, n: int, m: int, sssp: Path, ce: Path):
    out = subprocess.run([str(REFBIN / "ref_update"), str(graph), str(n), str(m), str(sssp), str(ce)], check=True,
                         capture_output=True, text=True).stdout
    dist = [0] * n
    parent = [0] * n
    rounds = {}
    for line in out.splitlines():
        f = line.split()
        if f[0].startswith("rounds"):
            rounds[f[0]] = int(f[1])
            continue
        i = int(f[0])
        dist[i] = int(f[1])
        parent[i] = int(f[2])
    return dist, parent, rounds


def updated_lines(edges, changes):
    dels = {(min(u, v), max(u, v), w) for (u, v, w, op) in changes if op == 0}
    lines = list(edges) + [(u, v, w) for (u, v, w, op) in changes if op == 1]
    return [(u, v, w) for (u, v, w) in lines if (min(u, v), max(u, v), w) not in dels]


def random_case(rng: np.random.Generator, n: int, m: int, wmax: int, n_ins: int, n_del: int, extras: bool):
    edges = []
    for _ in range(m):
        a, b = int(rng.integers(0, n)), int(rng.integers(0, n))
        if a == b:
            continue
        edges.append((a, b, int(rng.integers(0 if extras else 1, wmax + 1))))
    if extras:
        for _ in range(max(1, m // 20)):  # parallel edges, some with the same weight
            a, b, w = edges[int(rng.integers(0, len(edges)))]
            edges.append((b, a, w if rng.random() < 0.5 else int(rng.integers(0, wmax + 1))))
    changes = []
    for _ in range(n_ins):
        a, b = int(rng.integers(0, n)), int(rng.integers(0, n))
        if a == b:
            continue
        changes.append((a, b, int(rng.integers(0 if extras else 1, wmax + 1)), 1))
    for _ in range(n_del):
        a, b, w = edges[int(rng.integers(0, len(edges)))]
        changes.append((a, b, w, 0))
    if extras:
        # an insertion deleted again in the same batch, a deletion of an absent edge,
        # a deletion whose weight does not match, and an ignored op
        a, b, w, _ = changes[0]
        changes.append((b, a, w, 0))
        changes.append((0, n - 1, 7, 0))
        a, b, w = edges[1]
        changes.append((a, b, w + 1000, 0))
        changes.append((1, 2, 3, 5))
    order = rng.permutation(len(changes))
    return edges, [changes[i] for i in order]


def shaped_cases(rng: np.random.Generator):
    """Cases of a fixed shape: a long path with chords (a cut-off subtree deeper than the
    subtree walk's level limit), a star (a hub's edges deleted, leaves joined), the source's
    every edge deleted, a batch of ignored records only, and repeated records."""
    cases = []
    n = 300  # path 0-1-...-299 with a few chords; deleting (3, 4) cuts off ~290 levels, which
    # the chord (2, 60) reaches again from the middle
    edges = [(i, i + 1, int(rng.integers(1, 10))) for i in range(n - 1)]
    edges += [(int(a), int(a) + int(rng.integers(5, 40)), int(rng.integers(50, 200)))
              for a in rng.integers(0, n - 41, 12)]
    edges.append((2, 60, 150))
    changes = [(3, 4, edges[3][2], 0), (150, 151, edges[150][2], 0), (10, 200, 500, 1), (7, 9, 3, 1)]
    cases.append(("deep_path", n, edges, changes))
    n = 80  # star around 0, a few leaf-leaf edges
    edges = [(0, i, int(rng.integers(1, 20))) for i in range(1, n)]
    edges += [(int(a), int(b), int(rng.integers(1, 40))) for a, b in rng.integers(1, n, (30, 2)) if a != b]
    changes = [(0, i, edges[i - 1][2], 0) for i in range(1, n, 3)]
    changes += [(int(a), int(b), int(rng.integers(1, 40)), 1) for a, b in rng.integers(1, n, (20, 2)) if a != b]
    cases.append(("star_hub_deletions", n, edges, [changes[i] for i in rng.permutation(len(changes))]))
    n = 50  # every edge of the source deleted: everything else becomes unreachable
    edges = [(int(a), int(b), int(rng.integers(1, 30))) for a, b in rng.integers(0, n, (150, 2)) if a != b]
    changes = [(a, b, w, 0) for (a, b, w) in edges if a == 0 or b == 0]
    cases.append(("source_isolated", n, edges, changes))
    edges = [(int(a), int(b), int(rng.integers(1, 30))) for a, b in rng.integers(0, n, (150, 2)) if a != b]
    cases.append(("ignored_records_only", n, edges, [(1, 2, 3, 5), (4, 5, 6, 2), (7, 8, 9, -1)]))
    edges = [(int(a), int(b), int(rng.integers(1, 30))) for a, b in rng.integers(0, n, (150, 2)) if a != b]
    a, b, w = edges[5]
    c, d, x = edges[9]
    changes = [(a, b, w, 0), (b, a, w, 0), (a, b, w, 0), (1, 40, 4, 1), (40, 1, 4, 1), (1, 40, 4, 1), (c, d, x, 0)]
    cases.append(("repeated_records", n, edges, changes))
    return cases


def more_cases(rng: np.random.Generator):
    """A grid with cut edges and diagonal shortcuts (a high-diameter tree), a graph whose
    endpoints follow a skewed law (hubs) with hub-heavy changes, a cut-off subtree that an
    insertion of the same batch reattaches by a cheaper edge, and weights of 0 and 1 only with
    deletions of tree edges (zero-weight ties)."""
    cases = []
    side = 15  # 15 x 15 grid, id = r * 15 + c, weights 1..9
    n = side * side
    edges = [(r * side + c, r * side + c + 1, int(rng.integers(1, 10))) for r in range(side) for c in range(side - 1)]
    edges += [(r * side + c, (r + 1) * side + c, int(rng.integers(1, 10))) for r in range(side - 1) for c in range(side)]
    pick = rng.choice(len(edges), 20, replace=False)
    changes = [(edges[int(i)][0], edges[int(i)][1], edges[int(i)][2], 0) for i in pick]
    changes.append((0, 1, edges[0][2], 0))  # one of the source's two edges
    for _ in range(10):
        r, c = int(rng.integers(0, side - 1)), int(rng.integers(0, side - 1))
        changes.append((r * side + c, (r + 1) * side + c + 1, int(rng.integers(1, 12)), 1))
    cases.append(("grid_cuts", n, edges, [changes[i] for i in rng.permutation(len(changes))]))
    n = 512  # skewed endpoints: low ids are hubs
    def skewed():
        return int(n * rng.random() ** 3)
    edges = []
    while len(edges) < 2000:
        a, b = skewed(), skewed()
        if a != b:
            edges.append((a, b, int(rng.integers(1, 51))))
    changes = [(*edges[int(i)], 0) for i in rng.choice(len(edges), 100, replace=False)]
    while len(changes) < 200:
        a, b = skewed(), skewed()
        if a != b:
            changes.append((a, b, int(rng.integers(1, 51)), 1))
    cases.append(("skewed_hubs", n, edges, [changes[i] for i in rng.permutation(len(changes))]))
    n = 60  # path 0-...-59 (weights 5) with one long chord; cut at 10-11, reattached by 5-30 (w 1)
    edges = [(i, i + 1, 5) for i in range(n - 1)] + [(0, 45, 400)]
    changes = [(10, 11, 5, 0), (5, 30, 1, 1), (40, 41, 5, 0)]
    cases.append(("insert_reattaches", n, edges, changes))
    n = 40  # weights 0 and 1: equal-distance ties everywhere
    edges = [(int(a), int(b), int(rng.integers(0, 2))) for a, b in rng.integers(0, n, (140, 2)) if a != b]
    changes = [(a, b, w, 0) for (a, b, w) in edges[:25]]
    changes += [(int(a), int(b), int(rng.integers(0, 2)), 1) for a, b in rng.integers(0, n, (12, 2)) if a != b]
    cases.append(("weights_0_1", n, edges, [changes[i] for i in rng.permutation(len(changes))]))
    return cases


def make_case(tmp: Path, name: str, n: int, edges, changes, sssp_rows=None):
    g = tmp / f"{name}_graph.txt"
    s = tmp / f"{name}_SSSP.txt"
    c = tmp / f"{name}_cE.txt"
    u = tmp / f"{name}_updated.txt"
    write_lines(g, edges)
    write_lines(c, changes)
    if sssp_rows is None:
        par0, dist0 = run_seq(g, n)
        sssp_rows = [(i, par0[i], int(dist0[i])) for i in range(n)]
    write_lines(s, sssp_rows)
    upd = updated_lines(edges, changes)
    write_lines(u, upd)
    par1, dist1 = run_seq(u, n)
    rd, rp, rounds = run_ref_update(g, n, len(edges), s, c)
    return {
        "name": name,
        "n": n,
        "edges": [list(e) for e in edges],
        "changes": [list(x) for x in changes],
        "sssp_in": [list(r) for r in sssp_rows],
        "seq_after": {"parent": par1, "dist": [int(x) for x in dist1], "inf": 1000 * n},
        "ref_update": {"dist": rd, "parent": rp, "rounds": rounds},
    }


def main() -> int:
    if not os.environ.get("DSSSP_REFERENCE") or not (REF / "seqSSSPwithDist_undir.cpp").exists():
        print("set DSSSP_REFERENCE to the reference's source directory", file=sys.stderr)
        return 1
    build_ref()
    cases = []
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)
        sample_edges = [tuple(int(x) for x in l.split()[:3]) for l in (REF / "graph.txt").read_text().splitlines() if l.split()]
        sample_changes = [tuple(int(x) for x in l.split()[:4]) for l in (REF / "cE.txt").read_text().splitlines() if l.split()]
        sample_sssp = [tuple(int(x) for x in l.split()[:3]) for l in (REF / "SSSP.txt").read_text().splitlines() if l.split()]
        cases.append(make_case(tmp, "sample", 6, sample_edges, sample_changes, sample_sssp))
        rng = np.random.default_rng(20261203)
        specs = [
            ("er_small", 40, 120, 20, 10, 10, False),
            ("er_extras", 60, 200, 9, 15, 15, True),
            ("sparse_disconnected", 120, 100, 50, 20, 20, False),
            ("dense_weights0", 30, 250, 3, 20, 25, True),
            ("mid", 200, 700, 100, 40, 40, True),
            ("mid_delete_heavy", 200, 600, 30, 5, 120, False),
            ("mid_insert_heavy", 200, 500, 30, 120, 5, True),
        ]
        for name, n, m, wmax, ni, nd, extras in specs:
            edges, changes = random_case(rng, n, m, wmax, ni, nd, extras)
            cases.append(make_case(tmp, name, n, edges, changes))
        for name, n, edges, changes in shaped_cases(np.random.default_rng(20261204)):
            cases.append(make_case(tmp, name, n, edges, changes))
        for name, n, edges, changes in more_cases(np.random.default_rng(20261205)):
            cases.append(make_case(tmp, name, n, edges, changes))
    out = HERE / "golden.json"
    out.write_text(json.dumps({"generator": "tests/golden/make_golden.py", "cases": cases}, separators=(",", ":")))
    print(f"wrote {out} ({out.stat().st_size} bytes, {len(cases)} cases)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
