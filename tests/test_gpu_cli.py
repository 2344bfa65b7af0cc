"""The drop-in command line (SSSPmainForUndirected.cu's `op_main graph N M SSSP cE`) on the GPU:
the reference's sample files give the known answer, the stdout lines keep the reference's
wording, and --cache reads the binary images it wrote on the first run."""
import subprocess

import numpy as np
import pytest

import dynamicssspv2_gb300 as D
from oracle import pyoracle as O
from tests.common import case_arrays, golden_cases

pytestmark = pytest.mark.gpu


def write_case(tmp_path, case):
    u, v, w, ch = case_arrays(case)
    g = tmp_path / "graph.txt"
    g.write_text("".join(f"{a} {b} {c}\n" for a, b, c in zip(u.tolist(), v.tolist(), w.tolist())))
    s = tmp_path / "SSSP.txt"
    s.write_text("".join(f"{a} {b} {c}\n" for a, b, c in case["sssp_in"]))
    c = tmp_path / "cE.txt"
    D.write_changes(str(c), ch)
    return g, s, c, (u, v, w, ch)


def run_cli(*args):
    return subprocess.run([str(D.CLI_PATH), *map(str, args)], capture_output=True, text=True, timeout=300)


def test_sample_known_answer_and_stdout(tmp_path):
    case = next(c for c in golden_cases() if c["name"] == "sample")
    g, s, c, _ = write_case(tmp_path, case)
    out = tmp_path / "out.txt"
    r = run_cli(g, 6, 6, s, c, "--out", out)
    assert r.returncode == 0, r.stderr
    for line in ("Reading input graph completed", "Reading input changed edges data completed. totalInsertion:2",
                 "Total Time taken for SSSP update", "from GPU:"):
        assert line in r.stdout
    parent, dist, _ = D.read_sssp(str(out), 6)
    assert dist.tolist() == [0, 4, 6, 6, 4, 9]


def test_cache_round_trip_gives_the_same_tree(tmp_path):
    n = 3000
    u, v, w = D.gen_er(n, 12000, 1, 100, seed=21)
    d0, p0 = O.dijkstra(n, O.csr(n, u, v, w), 0)
    g = tmp_path / "graph.txt"
    g.write_text("".join(f"{a} {b} {c}\n" for a, b, c in zip(u.tolist(), v.tolist(), w.tolist())))
    s = tmp_path / "SSSP.txt"
    D.write_sssp(str(s), p0, d0)
    ch = D.gen_changes_ref(n, u, v, w, 800, 50, wlo=1, whi=99, seed=22)
    c = tmp_path / "cE.txt"
    D.write_changes(str(c), ch)
    outs = []
    for i, extra in enumerate(([], ["--cache"], ["--cache"], ["--cache", "--delta", "50"])):
        out = tmp_path / f"out{i}.txt"
        r = run_cli(g, n, len(u), s, c, "--out", out, *extra)
        assert r.returncode == 0, r.stderr
        assert "ignoring" not in r.stderr
        outs.append(D.read_sssp(str(out), n))
        if i == 1:
            assert (tmp_path / "graph.txt.dsssp.bin").exists() and (tmp_path / "SSSP.txt.dsssp.bin").exists()
    for parent, dist, _ in outs[1:]:
        assert np.array_equal(dist, outs[0][1])
    gr = O.updated_graph(n, u, v, w, ch)
    od, _ = O.dijkstra(n, gr, 0)
    assert np.array_equal(outs[0][1], od)
    assert O.validate(n, gr, 0, outs[3][1], outs[3][0]) == 0


def test_autotune_flag_tunes_then_reads_the_cache(tmp_path):
    """--autotune CACHE: the first run times the candidates on the batch (on snapshots) and
    writes the size class to CACHE, the second takes it from CACHE; both trees are exact."""
    n = 4000
    u, v, w = D.gen_er(n, 16000, 1, 100, seed=31)
    d0, p0 = O.dijkstra(n, O.csr(n, u, v, w), 0)
    g = tmp_path / "graph.txt"
    g.write_text("".join(f"{a} {b} {c}\n" for a, b, c in zip(u.tolist(), v.tolist(), w.tolist())))
    s = tmp_path / "SSSP.txt"
    D.write_sssp(str(s), p0, d0)
    ch = D.gen_changes(n, u, v, w, 400, 400, seed=32)
    c = tmp_path / "cE.txt"
    D.write_changes(str(c), ch)
    cache = tmp_path / "tune.txt"
    gr = O.updated_graph(n, u, v, w, ch)
    od, _ = O.dijkstra(n, gr, 0)
    for i, word in enumerate(("tuned", "cached settings")):
        out = tmp_path / f"out{i}.txt"
        r = run_cli(g, n, len(u), s, c, "--out", out, "--autotune", cache)
        assert r.returncode == 0, r.stderr
        assert f"autotune v12_e15_b10: {word}" in r.stderr, r.stderr
        parent, dist, _ = D.read_sssp(str(out), n)
        assert np.array_equal(dist, od)
        assert O.validate(n, gr, 0, dist, parent) == 0
    lines = [l for l in cache.read_text().splitlines() if not l.startswith("#")]
    assert len(lines) == 1 and lines[0].startswith("v12_e15_b10 ") and "small_deg=" in lines[0]
