"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg, never by the dsssp product.  See oracle.h for what each function restates.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"


def _load():
    if not LIB_PATH.exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    return C.CDLL(str(LIB_PATH))


_lib = _load()
_i32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64 = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_P = C.c_void_p

_lib.orc_updated_graph_nnz.restype = C.c_int64
_lib.orc_updated_graph_nnz.argtypes = [C.c_int32, C.c_int64, _i32, _i32, _i32, C.c_int64, _i32, _i32, _i32, _i32]
_lib.orc_updated_graph.restype = C.c_int64
_lib.orc_updated_graph.argtypes = [C.c_int32, C.c_int64, _i32, _i32, _i32, C.c_int64, _i32, _i32, _i32, _i32,
                                   _i64, _i32, _i32, _P]
_lib.orc_dijkstra.restype = C.c_int64
_lib.orc_dijkstra.argtypes = [C.c_int32, _i64, _i32, _i32, C.c_int32, C.c_int64, _i64, _i32]
_lib.orc_validate_tree.restype = C.c_int
_lib.orc_validate_tree.argtypes = [C.c_int32, _i64, _i32, _i32, C.c_int32, _i64, _i32, C.c_int64, C.c_char_p,
                                   C.c_int32]
_lib.orc_ref_update.restype = C.c_int
_lib.orc_ref_update.argtypes = [C.c_int32, C.c_int64, _i32, _i32, _i32, C.c_int64, _i32, _i32, _i32, _i32, _i32,
                                _i32, _i32, _i32, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
_lib.orc_read_sssp_semantics.restype = None
_lib.orc_read_sssp_semantics.argtypes = [C.c_int32, C.c_int64, _i32, _i32, _i32, _i32, _i32]

_lib.orc_gen_er.restype = C.c_int
_lib.orc_gen_er.argtypes = [C.c_int32, C.c_int64, C.c_int32, C.c_int32, C.c_uint64, _i32, _i32, _i32]
_lib.orc_gen_rmat.restype = C.c_int
_lib.orc_gen_rmat.argtypes = [C.c_int32, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32,
                              C.c_uint64, _i32, _i32, _i32]
_lib.orc_max_degree_vertex.restype = C.c_int32
_lib.orc_max_degree_vertex.argtypes = [C.c_int32, C.c_int64, _i32, _i32]
_lib.orc_gen_changes.restype = C.c_int
_lib.orc_gen_changes.argtypes = [C.c_int32, C.c_int64, _i32, _i32, _i32, C.c_int64, C.c_int64, C.c_int32, C.c_int32,
                                 C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32, C.c_uint64, _i32, _i32,
                                 _i32, _i32]

EXACT_INF = (1 << 62)

CHANGE_DTYPE = np.dtype([("u", "<i4"), ("v", "<i4"), ("w", "<i4"), ("op", "<i4")])


def gen_er(n, m, wlo=1, whi=100, seed=0):
    """Erdos-Renyi edge list of the library's generator (same streams), on the CPU."""
    u, v, w = (np.empty(m, np.int32) for _ in range(3))
    if _lib.orc_gen_er(n, m, wlo, whi, seed, u, v, w) != 0:
        raise ValueError("gen_er: bad arguments")
    return u, v, w


def gen_rmat(scale, m, a=0.57, b=0.19, c=0.19, wlo=1, whi=100, seed=0):
    u, v, w = (np.empty(m, np.int32) for _ in range(3))
    if _lib.orc_gen_rmat(scale, m, a, b, c, wlo, whi, seed, u, v, w) != 0:
        raise ValueError("gen_rmat: bad arguments")
    return u, v, w


def max_degree_vertex(n, u, v):
    return int(_lib.orc_max_degree_vertex(n, len(u), _a32(u), _a32(v)))


def gen_changes(n, u, v, w, n_ins, n_del, kind=0, scale=0, p0=0.0, p1=0.0, p2=0.0, wlo=1, whi=100, seed=0):
    """A change batch of the library's dsssp_gen_changes (uniform or RMAT insertions)."""
    k = n_ins + n_del
    cu, cv, cw, cop = (np.empty(k, np.int32) for _ in range(4))
    if _lib.orc_gen_changes(n, len(u), _a32(u), _a32(v), _a32(w), n_ins, n_del, kind, scale, p0, p1, p2, wlo, whi,
                            seed, cu, cv, cw, cop) != 0:
        raise ValueError("gen_changes: bad arguments or too few new pairs")
    out = np.empty(k, CHANGE_DTYPE)
    out["u"], out["v"], out["w"], out["op"] = cu, cv, cw, cop
    return out


def _a32(x):
    return np.ascontiguousarray(x, np.int32)


def _split_changes(changes):
    if changes is None or len(changes) == 0:
        z = np.zeros(0, np.int32)
        return z, z, z, z
    return _a32(changes["u"]), _a32(changes["v"]), _a32(changes["w"]), _a32(changes["op"])


class CSR:
    def __init__(self, off, col, wt):
        self.off, self.col, self.wt = off, col, wt


def updated_graph(n, u, v, w, changes=None, return_kept=False):
    """CSR of the graph after the batch (reference batch semantics)."""
    u, v, w = _a32(u), _a32(v), _a32(w)
    cu, cv, cw, cop = _split_changes(changes)
    nnz = _lib.orc_updated_graph_nnz(n, len(u), u, v, w, len(cu), cu, cv, cw, cop)
    if nnz < 0:
        raise ValueError("vertex id out of range")
    off = np.zeros(n + 1, np.int64)
    col = np.zeros(max(nnz, 1), np.int32)
    wt = np.zeros(max(nnz, 1), np.int32)
    kept = np.zeros(len(u) + len(cu) + 1, np.uint8)
    _lib.orc_updated_graph(n, len(u), u, v, w, len(cu), cu, cv, cw, cop, off, col, wt, kept.ctypes.data)
    g = CSR(off, col[:nnz], wt[:nnz])
    if return_kept:
        return g, kept
    return g


def csr(n, u, v, w):
    return updated_graph(n, u, v, w, None)


def dijkstra(n, g: CSR, src, inf_cap=None):
    """Sequential Dijkstra with the reference's semantics; returns (dist int64, parent int32).
    inf_cap None = exact (no 1000*N cap); unreachable vertices get dist -1 then."""
    exact = inf_cap is None
    cap = EXACT_INF if exact else int(inf_cap)
    dist = np.zeros(n, np.int64)
    parent = np.zeros(n, np.int32)
    col = g.col if len(g.col) else np.zeros(1, np.int32)
    wt = g.wt if len(g.wt) else np.zeros(1, np.int32)
    _lib.orc_dijkstra(n, g.off, col, wt, int(src), cap, dist, parent)
    if exact:
        dist[parent == -1] = -1
    return dist, parent


def validate(n, g: CSR, src, dist, parent, unreach=-1):
    """0 if (dist, parent) is a valid shortest-path tree of g, else (code, message)."""
    buf = C.create_string_buffer(256)
    col = g.col if len(g.col) else np.zeros(1, np.int32)
    wt = g.wt if len(g.wt) else np.zeros(1, np.int32)
    rc = _lib.orc_validate_tree(n, g.off, col, wt, int(src), np.ascontiguousarray(dist, np.int64),
                                _a32(parent), int(unreach), buf, 256)
    return 0 if rc == 0 else (rc, buf.value.decode())


def read_sssp_semantics(n, node, par, dist):
    out_p = np.zeros(n, np.int32)
    out_d = np.zeros(n, np.int32)
    node, par, dist = _a32(node), _a32(par), _a32(dist)
    _lib.orc_read_sssp_semantics(n, len(node), node, par, dist, out_p, out_d)
    return out_p, out_d


def ref_update(n, u, v, w, changes, in_parent, in_dist):
    """The reference GPU update replayed one thread at a time; returns (Dist, Parent, rounds)."""
    u, v, w = _a32(u), _a32(v), _a32(w)
    cu, cv, cw, cop = _split_changes(changes)
    od = np.zeros(n, np.int32)
    op = np.zeros(n, np.int32)
    r1, r2 = C.c_int64(), C.c_int64()
    rc = _lib.orc_ref_update(n, len(u), u, v, w, len(cu), cu, cv, cw, cop, _a32(in_parent), _a32(in_dist), od, op,
                             C.byref(r1), C.byref(r2))
    if rc != 0:
        raise RuntimeError(f"orc_ref_update failed: {rc}")
    return od, op, (r1.value, r2.value)


def dijkstra_after(n, u, v, w, changes, src):
    """Exact shortest-path distances of the graph after the batch."""
    g = updated_graph(n, u, v, w, changes)
    return dijkstra(n, g, src)
