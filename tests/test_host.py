"""Host-side parts of the library, CPU only: the C ABI's exported symbols, the seeded
generators, the reference text formats, and the drop-in command line's argument handling."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import dynamicssspv2_gb300 as D

ROOT = Path(__file__).resolve().parents[1]


def header_functions():
    text = (ROOT / "include" / "dsssp.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dsssp_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_function_is_exported():
    names = header_functions()
    assert len(names) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", str(D.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r" T (dsssp_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    for n in names:
        assert hasattr(D._lib, n)
    assert set(D.EXPORTED) <= set(names)


def test_errors_have_messages():
    for code in range(0, -13, -1):
        assert D._lib.dsssp_strerror(code).decode() != "unknown error"
    assert D._lib.dsssp_strerror(-99).decode() == "unknown error"


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_no_device_is_reported():
    with pytest.raises(D.DsssspError) as e:
        D.Graph(4, [0, 1], [1, 2], [1, 1])
    assert e.value.code == D.E_NO_DEVICE


# ---- generators ---------------------------------------------------------------------------

def _keys(u, v):
    return np.minimum(u, v).astype(np.int64) * (1 << 32) + np.maximum(u, v)


def test_er_exact_distinct_and_deterministic():
    u, v, w = D.gen_er(1000, 5000, 1, 100, 7)
    assert len(u) == 5000
    assert (u != v).all()
    assert len(np.unique(_keys(u, v))) == 5000
    assert w.min() >= 1 and w.max() <= 100
    u2, v2, w2 = D.gen_er(1000, 5000, 1, 100, 7)
    assert (u == u2).all() and (v == v2).all() and (w == w2).all()
    u3, _, _ = D.gen_er(1000, 5000, 1, 100, 8)
    assert not (u == u3).all()


def test_rmat_is_skewed_and_exact():
    u, v, w = D.gen_rmat(12, 30000, seed=3)
    assert len(np.unique(_keys(u, v))) == 30000 and (u != v).all()
    assert u.max() < 4096 and v.max() < 4096
    deg = np.bincount(np.concatenate([u, v]), minlength=4096)
    assert deg.max() > 20 * deg.mean()  # hubs
    assert D.max_degree_vertex(4096, u, v) == int(np.argmax(deg))


def test_grid_counts():
    rows, cols = 64, 50
    u, v, w = D.gen_grid(rows, cols, 0.05, 30, 1, 1000, 1)
    e4 = rows * (cols - 1) + (rows - 1) * cols
    assert len(u) == e4 - int(0.05 * e4) + 30
    ru, cu, rv, cv = u // cols, u % cols, v // cols, v % cols
    assert (np.maximum(abs(ru - rv), abs(cu - cv)) == 1).all()
    assert len(np.unique(_keys(u, v))) == len(u)


@pytest.mark.parametrize("kind", [D.INS_UNIFORM, D.INS_RMAT, D.INS_LOCAL])
def test_change_batches(kind):
    if kind == D.INS_LOCAL:
        n, cols = 40 * 40, 40
        u, v, w = D.gen_grid(40, 40, 0.0, 0, 1, 9, 2)
        ch = D.gen_changes(n, u, v, w, 200, 300, kind, cols, 2.0, 0, 0, 1, 9, seed=5)
    else:
        n = 4096
        u, v, w = D.gen_rmat(12, 20000, seed=2) if kind == D.INS_RMAT else D.gen_er(n, 20000, 1, 9, 2)
        ch = D.gen_changes(n, u, v, w, 200, 300, kind, 12, 0.57, 0.19, 0.19, 1, 9, seed=5)
    assert len(ch) == 500
    ins, dels = ch[ch["op"] == 1], ch[ch["op"] == 0]
    assert len(ins) == 200 and len(dels) == 300
    existing = set(_keys(u, v).tolist())
    ik = _keys(ins["u"], ins["v"])
    assert len(set(ik.tolist())) == 200 and not (set(ik.tolist()) & existing)
    assert (ins["u"] != ins["v"]).all()
    lines = set(zip(u.tolist(), v.tolist(), w.tolist()))
    assert all((a, b, c) in lines for a, b, c in zip(dels["u"].tolist(), dels["v"].tolist(), dels["w"].tolist()))
    assert len(set(zip(dels["u"].tolist(), dels["v"].tolist()))) == 300
    if kind == D.INS_LOCAL:
        assert (np.maximum(abs(ins["u"] // cols - ins["v"] // cols), abs(ins["u"] % cols - ins["v"] % cols)) <= 2).all()
    assert not (ch["op"][:200] == 1).all()  # shuffled


# ---- text formats -------------------------------------------------------------------------

def test_graph_and_change_files_round_trip(tmp_path):
    g = tmp_path / "graph.txt"
    g.write_text("0 1 2\n0  2 6 \n\n1 3 2\nbad line\n1 4\n4 2 2\n")
    u, v, w = D.read_graph(str(g), 6)
    assert list(zip(u, v, w)) == [(0, 1, 2), (0, 2, 6), (1, 3, 2), (4, 2, 2)]  # short lines skipped
    c = tmp_path / "cE.txt"
    c.write_text("0 1 2 0\n0  4 4 1 \n1 4 0 1\n3 2 1 7\n")  # the reference's generator writes double spaces
    ch = D.read_changes(str(c), 6)
    assert ch.tolist() == [(0, 1, 2, 0), (0, 4, 4, 1), (1, 4, 0, 1), (3, 2, 1, 7)]


def test_out_of_range_vertex_and_missing_file(tmp_path):
    g = tmp_path / "graph.txt"
    g.write_text("0 1 2\n0 9 1\n")
    with pytest.raises(D.DsssspError) as e:
        D.read_graph(str(g), 6)
    assert e.value.code == D.E_BAD_VERTEX
    with pytest.raises(D.DsssspError) as e:
        D.read_graph(str(tmp_path / "nope.txt"), 6)
    assert e.value.code == D.E_IO
    c = tmp_path / "c.txt"
    c.write_text("0 7 1 1\n")
    with pytest.raises(D.DsssspError) as e:
        D.read_changes(str(c), 6)
    assert e.value.code == D.E_BAD_VERTEX
    c.write_text("0 7 1 3\n")  # ignored op: not checked, as in the reference
    assert len(D.read_changes(str(c), 6)) == 1
    # every out-of-range id is reported, -1 and ids beyond 64 bits included
    for text, reader in (("-1 2 3\n", D.read_graph), ("2 -1 3\n", D.read_graph),
                         ("1 99999999999999999999999 3\n", D.read_graph), ("-1 2 3 0\n", D.read_changes),
                         ("0 -1 3 1\n", D.read_changes), ("-1 0 0\n", D.read_sssp)):
        f = tmp_path / "bad.txt"
        f.write_text("0 1 2 1\n" + text)
        with pytest.raises(D.DsssspError) as e:
            reader(str(f), 6)
        assert e.value.code == D.E_BAD_VERTEX, (text, reader)


def test_sssp_file_semantics(tmp_path):
    """read_SSSP (all_structure_undir.cuh:133-171): gaps and parent -1 are unreachable; the
    reference's Dijkstra writes distances with cout (%g-like), which is accepted here."""
    s = tmp_path / "SSSP.txt"
    s.write_text("0 0 0\n1 0 2\n3 1 1.2e+06\n4 -1 6000\n")
    parent, dist, lossy = D.read_sssp(str(s), 6)
    assert parent.tolist() == [0, 0, -1, 1, -1, -1]
    assert dist.tolist() == [0, 2, -1, 1200000, -1, -1]
    assert lossy == 1


def test_sssp_write_read_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    n = 1000
    parent = rng.integers(-1, n, n).astype(np.int32)
    dist = np.where(parent == -1, -1, rng.integers(0, 1 << 31, n)).astype(np.int64)
    out = tmp_path / "out.txt"
    D.write_sssp(str(out), parent, dist)
    p2, d2, lossy = D.read_sssp(str(out), n)
    assert (p2 == parent).all() and (d2 == dist).all() and lossy == 0


def test_large_file_parses_in_parallel_chunks(tmp_path):
    u, v, w = D.gen_er(50000, 300000, 1, 100, 3)
    g = tmp_path / "big.txt"
    with open(g, "w") as f:
        f.write("".join(f"{a} {b} {c}\n" for a, b, c in zip(u.tolist(), v.tolist(), w.tolist())))
    u2, v2, w2 = D.read_graph(str(g), 50000)
    assert (u2 == u).all() and (v2 == v).all() and (w2 == w).all()


# ---- command line -----------------------------------------------------------------------------

def test_cli_usage_and_errors(tmp_path):
    r = subprocess.run([str(D.CLI_PATH)], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([str(D.CLI_PATH), str(tmp_path / "nope.txt"), "6", "6", "x", "y"], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "reading the graph" in r.stderr
    assert r.stdout.startswith("Reading input graph...")
    g = tmp_path / "g.txt"
    g.write_text("0 1 2\n")
    for args, msg in ((["abc", "1"], "number_of_nodes"), (["99999999999", "1"], "number_of_nodes"),
                      (["0", "1"], "number_of_nodes"), (["3", "-1"], "number_of_edges"), (["3", "2x"], "number_of_edges"),
                      (["3", "1", "--delta", "x"], "bad option --delta"), (["3", "1", "--out"], "bad option --out"),
                      (["3", "1", "--device", "7b"], "bad option --device")):
        r = subprocess.run([str(D.CLI_PATH), str(g), args[0], args[1], "s", "c"] + args[2:], capture_output=True,
                           text=True)
        assert r.returncode == 2 and msg in r.stderr, (args, r.stderr)


# ---- binary cache, the reference generator's format and sampling -----------------------------

def test_graph_binary_round_trip_and_rejections(tmp_path):
    u, v, w = D.gen_rmat(12, 30001, seed=4)  # odd edge count: a padded checksum tail word
    path = tmp_path / "g.bin"
    D.write_graph_binary(str(path), 1 << 12, u, v, w)
    u2, v2, w2 = D.read_graph_binary(str(path), 1 << 12)
    assert (u2 == u).all() and (v2 == v).all() and (w2 == w).all()
    with pytest.raises(D.DsssspError) as e:  # other vertex count than the cache holds
        D.read_graph_binary(str(path), 1 << 11)
    assert e.value.code == D.E_IO
    data = bytearray(path.read_bytes())
    data[32 + 4 * 12345] ^= 0x10  # one flipped payload bit
    bad = tmp_path / "bad.bin"
    bad.write_bytes(bytes(data))
    with pytest.raises(D.DsssspError) as e:
        D.read_graph_binary(str(bad), 1 << 12)
    assert e.value.code == D.E_IO and "checksum" in str(e.value)
    bad.write_bytes(path.read_bytes()[:-8])  # truncated
    with pytest.raises(D.DsssspError) as e:
        D.read_graph_binary(str(bad), 1 << 12)
    assert e.value.code == D.E_IO
    txt = tmp_path / "g.txt"
    txt.write_text("0 1 2\n")
    with pytest.raises(D.DsssspError) as e:  # a text file is not a cache
        D.read_graph_binary(str(txt), 6)
    assert e.value.code == D.E_IO
    empty = tmp_path / "e.bin"
    D.write_graph_binary(str(empty), 5, [], [], [])
    assert all(len(a) == 0 for a in D.read_graph_binary(str(empty), 5))
    # a header whose edge count disagrees with the file (here: ~10^18 edges) is refused before
    # anything is allocated for it; so are trailing bytes
    data = bytearray(path.read_bytes())
    data[16:24] = (0x0C00000000000FA0).to_bytes(8, "little")
    bad.write_bytes(bytes(data))
    with pytest.raises(D.DsssspError) as e:
        D.read_graph_binary(str(bad), 1 << 12)
    assert e.value.code == D.E_IO and "file size" in str(e.value)
    bad.write_bytes(path.read_bytes() + b"\0" * 12)
    with pytest.raises(D.DsssspError) as e:
        D.read_graph_binary(str(bad), 1 << 12)
    assert e.value.code == D.E_IO


def test_tree_binary_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    n = 777
    parent = rng.integers(-1, n, n).astype(np.int32)
    dist = np.where(parent == -1, -1, rng.integers(0, 1 << 40, n)).astype(np.int64)
    path = tmp_path / "t.bin"
    D.write_sssp_binary(str(path), parent, dist)
    p2, d2 = D.read_sssp_binary(str(path), n)
    assert (p2 == parent).all() and (d2 == dist).all()
    with pytest.raises(D.DsssspError):
        D.read_sssp_binary(str(path), n + 1)
    with pytest.raises(D.DsssspError):  # a graph image is not a tree image
        D.write_graph_binary(str(path), n, [0], [1], [2])
        D.read_sssp_binary(str(path), n)


def test_changes_file_in_the_reference_generator_format(tmp_path):
    ch = D.make_changes([0, 0, 1], [1, 4, 4], [2, 4, 0], [0, 1, 1])
    path = tmp_path / "cE.txt"
    D.write_changes(str(path), ch)
    # createChangedEdges.cpp:104 ("%d  %d %d 1 \n") and :116 ("%d %d %d 0 \n")
    assert path.read_text() == "0 1 2 0 \n0  4 4 1 \n1  4 0 1 \n"
    assert D.read_changes(str(path), 6).tolist() == ch.tolist()
    big = D.gen_changes(1000, *D.gen_er(1000, 5000, seed=2), 300, 300, seed=3)
    D.write_changes(str(path), big)
    assert D.read_changes(str(path), 1000).tolist() == big.tolist()


def test_reference_style_change_sampling():
    n = 500
    u, v, w = D.gen_er(n, 2000, 1, 100, seed=7)
    ch = D.gen_changes_ref(n, u, v, w, 5000, 30, seed=11)
    ins, dels = ch[ch["op"] == 1], ch[ch["op"] == 0]
    assert len(ch) == 5000 and len(ins) == int(5000 * 0.30) and len(dels) == 5000 - len(ins)
    assert (ins["u"] < ins["v"]).all() and (ins["w"] >= 0).all() and (ins["w"] <= 99).all()
    assert (ins["w"] == 0).any()  # the reference's rand() % 100 includes weight 0
    lines = set(zip(u.tolist(), v.tolist(), w.tolist()))
    assert all(t in lines for t in zip(dels["u"].tolist(), dels["v"].tolist(), dels["w"].tolist()))
    assert len(set(zip(dels["u"].tolist(), dels["v"].tolist()))) < len(dels)  # with replacement
    first = ch["op"][:200]
    assert 0 < first.sum() < 200  # coin-flip interleaving, not blocks
    again = D.gen_changes_ref(n, u, v, w, 5000, 30, seed=11)
    assert again.tolist() == ch.tolist()
    assert D.gen_changes_ref(n, u, v, w, 5000, 30, seed=12).tolist() != ch.tolist()


def test_bench_reads_the_committed_profiles():
    """bench.py's roofline reads ncu figures from profiles/: the update kernel's DRAM bytes per
    launch and the front kernels' (their bandwidth = bytes / live time, as a fraction of the
    peak)."""
    import bench

    traffic = bench.profiled_traffic("rmat22")
    assert traffic is not None and 1e8 < traffic < 1e9
    assert bench.profiled_value("k_update", "no_such_workload", "dram_bytes_per_launch") is None

    class S:  # stand-in for the engine's stats of two batches
        def __init__(self, d, a):
            self.t_delete_ms, self.t_append_ms = d, a

    out = bench.front_roofline("rmat22", [S(0.14, 0.08), S(0.16, 0.10)], 6771.1)
    dele, app = out["k_delete"], out["k_append"]
    assert abs(dele["ms_per_launch"] - 0.15) < 1e-12 and abs(app["ms_per_launch"] - 0.09) < 1e-12
    assert abs(dele["achieved_dram_gbs"] - dele["traffic"] / 0.15e-3 / 1e9) < 1e-6
    assert abs(dele["frac_dram"] - dele["achieved_dram_gbs"] / 6771.1) < 1e-12
    assert 0 < app["frac_dram"] < dele["frac_dram"] < 1


def test_serving_and_tuning_helpers():
    """Host-side helpers of the batching and serving layers: request summaries (p50/p99,
    refused and failed requests), random tenant batches, the autotuner's size classes, near-far
    candidates and cache file, and the footprint estimate's growth."""
    from dynamicssspv2_gb300.autotune import candidates, size_class
    from dynamicssspv2_gb300.serve import Request, Tenant, estimate_footprint, random_batch, summarize

    ch = np.zeros(10, D.CHANGE_DTYPE)
    reqs = [Request(0, 0.001 * i, ch, epoch=i // 2, done=0.001 * i + 0.002) for i in range(10)]
    reqs.append(Request(1, 0.0, ch, refused=True))
    reqs.append(Request(0, 0.0, ch, error="bad vertex"))
    s = summarize(reqs)
    assert s["requests"] == 12 and s["served"] == 10 and s["refused"] == 1 and s["failed"] == 1
    assert s["changes"] == 100 and abs(s["p50_ms"] - 2.0) < 1e-9 and abs(s["p99_ms"] - 2.0) < 1e-9
    assert s["epochs"] == 5 and s["mean_requests_per_epoch"] == 2.0
    assert summarize([])["p99_ms"] is None

    u, v, w = D.gen_er(100, 300, 1, 9, seed=2)
    t = Tenant("t", 100, u, v, w)
    b = random_batch(np.random.default_rng(3), t, 50, ins_frac=0.4)
    assert len(b) == 50 and (b["op"] == 1).sum() == 20 and (b["u"] != b["v"])[b["op"] == 1].all()
    dels = b[b["op"] == 0]
    lines = set(zip(u.tolist(), v.tolist(), w.tolist()))
    assert all((x, y, z) in lines for x, y, z in zip(dels["u"].tolist(), dels["v"].tolist(), dels["w"].tolist()))

    assert size_class(1 << 20, 1 << 24, 1000) == "v20_e24_b10"
    wbar = float(np.mean(b["w"]))
    base = D.default_opts()
    cands = candidates(base, b)
    # the fixed candidates (the defaults first), then two near-far widths from the batch's mean weight
    assert len(cands) == 12 and cands[0].small_deg == base.small_deg and cands[0].delta == base.delta
    assert [c.delta for c in cands[-2:]] == [max(1, int(np.floor(f * wbar + 0.5))) for f in (8.0, 96.0)]
    assert {c.solo_waves for c in cands} == {0, 2, 4} and {c.bfs_levels for c in cands} == {0, 8, 48}
    assert len(candidates(base, np.zeros(0, D.CHANGE_DTYPE))) == 10

    assert estimate_footprint(1000, 4000) < estimate_footprint(2000, 4000) < estimate_footprint(2000, 8000)


def test_generators_refuse_impossible_requests():
    """More distinct pairs than exist, or a distribution that keeps drawing the same pair, is
    an error rather than an endless draw."""
    for call in (lambda: D.gen_er(10, 46, 1, 5, 1),
                 lambda: D.gen_rmat(2, 7, 0.57, 0.19, 0.19, 1, 10, 2),
                 lambda: D.gen_rmat(1, 2, 0.57, 0.19, 0.19, 1, 10, 2),
                 lambda: D.gen_rmat(3, 10, 1.0, 0.0, 0.0, 1, 10, 2),   # every draw is the self-loop (0, 0)
                 lambda: D.gen_grid(3, 3, 0.0, 100, 1, 5, 3)):         # 8 diagonals exist
        with pytest.raises(D.DsssspError) as e:
            call()
        assert e.value.code == D.E_INVAL
    assert len(D.gen_rmat(2, 6, 0.57, 0.19, 0.19, 1, 10, 2)[0]) == 6   # every pair of 4 vertices
    assert len(D.gen_grid(3, 3, 0.0, 8, 1, 5, 3)[0]) == 12 + 8
    u, v, w = D.gen_er(20, 60, 1, 9, seed=1)
    with pytest.raises(D.DsssspError):
        D.gen_changes(20, u, v, w, 500, 0)   # only 130 new pairs
    assert len(D.gen_changes(20, u, v, w, 0, 0)) == 0


def test_noalloc_refuses_bad_pointers_before_any_launch():
    """dsssp_sssp_noalloc checks its pointers on the host: NULL or misaligned (d_row_off,
    d_adj, d_dist to 8 bytes, d_parent to 4) gives DSSSP_E_INVAL before any CUDA call, so
    these never reach a device (none is needed here)."""
    good8, good4 = 1 << 20, 1 << 20
    cases = [
        (0, good8, good4, good8),            # NULL row offsets
        (good8 + 4, good8, good4, good8),    # row offsets on 4 bytes
        (good8, good8 + 4, good4, good8),    # adjacency on 4 bytes
        (good8, good8, good4 + 2, good8),    # parents on 2 bytes
        (good8, good8, good4, good8 + 4),    # distances on 4 bytes
        (good8, good8, 0, good8),            # NULL parents
    ]
    for off, adj, par, dist in cases:
        with pytest.raises(D.DsssspError) as e:
            D.sssp_noalloc(100, 10, off, adj, 0, par, dist)
        assert e.value.code == D.E_INVAL


def test_abi_struct_sizes_match_the_binding():
    """dsssp_abi_sizes: the library's struct sizes equal the ctypes layouts (the binding
    refuses to import otherwise), and the fields appended last sit at the end."""
    import ctypes as C

    import dynamicssspv2_gb300 as D
    from dynamicssspv2_gb300.autotune import TuneResult

    assert D.abi_sizes() == [C.sizeof(D.Opts), C.sizeof(D.Stats), C.sizeof(D.ServerOpts), C.sizeof(D.RequestInfo),
                             C.sizeof(TuneResult)]
    assert D.Stats.t_seed_ms.offset + 8 == C.sizeof(D.Stats)
    out = (C.c_size_t * 2)()
    assert D._lib.dsssp_abi_sizes(out, 2) == 2 and list(out) == D.abi_sizes()[:2]


def test_tree_reads_refuse_a_null_graph_on_the_host():
    """The tree reads and the asynchronous read's wait refuse a NULL graph with DSSSP_E_INVAL
    before touching a device; dsssp_abi_sizes writes at most cap sizes."""
    import ctypes as C

    import dynamicssspv2_gb300 as D

    buf = (C.c_int32 * 4)()
    assert D._lib.dsssp_tree_read32(None, buf, buf) == D.E_INVAL
    assert D._lib.dsssp_tree_read32_async(None, buf, buf) == D.E_INVAL
    assert D._lib.dsssp_tree_read_wait(None) == D.E_INVAL
    assert D._lib.dsssp_tree_read(None, buf, buf) == D.E_INVAL
    sizes = (C.c_size_t * 1)()
    assert D._lib.dsssp_abi_sizes(sizes, 1) == 1 and sizes[0] == C.sizeof(D.Opts)
    assert D._lib.dsssp_abi_sizes(None, 5) == 0


def test_graph_and_change_readers_follow_the_reference_sscanf(tmp_path):
    """The graph and change readers take each field like the reference's sscanf("%d ...")
    (all_structure_undir.cuh:89-126, 178-198): whitespace of any kind between fields, a sign,
    the integer prefix of a token ("2.5" is 2), anything after the last field ignored; a line
    with fewer fields is skipped.  Files of several MB are parsed in parallel chunks, in order."""
    rng = np.random.default_rng(5)
    n = 1000
    seps = [" ", "  ", "\t", " \t "]
    ends = ["\n", "\r\n", " \n"]
    for nf, reader in ((3, D.read_graph), (4, D.read_changes)):
        lines, want = [], []
        for _ in range(220000):
            kind = int(rng.integers(0, 8))
            vals = [int(rng.integers(0, n)), int(rng.integers(0, n)), int(rng.integers(0, 100)), int(rng.integers(0, 2))][:nf]
            s = [seps[int(rng.integers(4))] for _ in range(nf)]
            end = ends[int(rng.integers(3))]
            body = "".join(f"{s[i - 1] if i else ''}{x}" for i, x in enumerate(vals))
            if kind == 0:  # one field short: skipped
                line = "".join(f"{s[i - 1] if i else ''}{x}" for i, x in enumerate(vals[:-1])) + end
            elif kind == 1:  # decimals in the last field: its integer prefix
                line = body + f".{int(rng.integers(0, 10))}" + end
                want.append(tuple(vals))
            elif kind == 2:  # junk and more numbers after the last field: ignored
                line = body + "abc 7 8" + end
                want.append(tuple(vals))
            elif kind == 3:  # a decimal in the second field: its remainder is not a number, skipped
                line = f"{vals[0]}{s[1]}{vals[1]}.5" + "".join(f"{s[i]}{vals[i]}" for i in range(2, nf)) + end
            elif kind == 4:  # blank
                line = end
            elif kind == 5:  # explicit sign
                line = "+" + body + end
                want.append(tuple(vals))
            else:  # leading whitespace
                line = s[0] + body + end
                want.append(tuple(vals))
            lines.append(line)
        f = tmp_path / f"fields{nf}.txt"
        f.write_text("".join(lines))
        assert f.stat().st_size > 2 << 20  # several parallel chunks
        got = reader(str(f), n)
        rows = list(zip(*got[:3])) if nf == 3 else [tuple(r) for r in got.tolist()]
        assert rows == want
