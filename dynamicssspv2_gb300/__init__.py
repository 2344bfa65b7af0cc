"""GB300-native dynamic single-source shortest paths (drop-in for the update path of
ArindamK92/DynamicSSSPv2).

The engine lives in the in-tree C ABI library ``_lib/libdsssp.so`` (include/dsssp.h); this
module binds it with ctypes.  There is no CPU fallback: importing the package fails if the
library has not been built (``python dynamicssspv2_gb300/_build.py``), and every engine call
needs a CUDA device.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libdsssp.so"
CLI_PATH = _PKG / "_lib" / "dsssp_main"

if not LIB_PATH.exists():
    raise ImportError(
        f"{LIB_PATH} is missing: build it with `python dynamicssspv2_gb300/_build.py` "
        "(the engine has no CPU fallback)"
    )

_lib = C.CDLL(str(LIB_PATH))

OK = 0
E_INVAL, E_OOM, E_BAD_VERTEX, E_CUDA, E_NO_CONVERGENCE, E_TIMEOUT = -1, -2, -3, -4, -5, -6
E_BAD_TREE, E_OVERFLOW, E_IO, E_BAD_WEIGHT, E_NO_DEVICE, E_COOP = -7, -8, -9, -10, -11, -12
UNREACHABLE = -1
UNREACHABLE32 = 0xFFFFFFFF
INS_UNIFORM, INS_RMAT, INS_LOCAL = 0, 1, 2

CHANGE_DTYPE = np.dtype([("u", "<i4"), ("v", "<i4"), ("w", "<i4"), ("op", "<i4")])


class DsssspError(RuntimeError):
    def __init__(self, code: int, what: str):
        self.code = code
        msg = _lib.dsssp_last_error().decode(errors="replace")
        super().__init__(f"{what}: {_lib.dsssp_strerror(code).decode()} ({code}): {msg}")


class Opts(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("slack_pct", C.c_int32),
        ("slack_min", C.c_int32),
        ("small_deg", C.c_int32),
        ("large_deg", C.c_int32),
        ("chunk", C.c_int32),
        ("bfs_levels", C.c_int32),
        ("block", C.c_int32),
        ("ctas_per_sm", C.c_int32),
        ("timing", C.c_int32),
        ("max_rounds", C.c_int64),
        ("spare_pct", C.c_int32),
        ("delta", C.c_int32),
        ("launch_graph", C.c_int32),
        ("recover", C.c_int32),
        ("warp_agg", C.c_int32),
        ("solo_waves", C.c_int32),
        ("auto_rounds", C.c_int32),
        ("group_ctas", C.c_int32),
        ("group_waves", C.c_int32),
    ]


class Stats(C.Structure):
    _fields_ = [
        (name, C.c_int64)
        for name in (
            "n_ins", "n_del", "n_ignored", "n_roots", "n_invalidated", "inv_levels", "pj_passes", "rounds",
            "frontier_total", "edges_relaxed", "edges_inval", "del_probed", "updates", "overflow_entries", "repacks",
            "n_killed", "work_items",
        )
    ] + [
        (name, C.c_double)
        for name in ("t_step1_ms", "t_inval_ms", "t_relax_ms", "t_update_ms", "t_total_ms", "bytes_alg",
                     "bytes_alg_update")
    ] + [("advances", C.c_int64), ("tombstoned", C.c_int64), ("graph_launch", C.c_int64),
         ("bytes_engine_update", C.c_double), ("t_delete_ms", C.c_double), ("t_append_ms", C.c_double),
         ("recovered_from", C.c_int64), ("t_recompute_ms", C.c_double), ("t_seed_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_chgp = np.ctypeslib.ndpointer(dtype=CHANGE_DTYPE, flags="C_CONTIGUOUS")
_P = C.c_void_p


def _sig(name, restype, *argtypes):
    f = getattr(_lib, name)
    f.restype = restype
    f.argtypes = list(argtypes)
    return f


_sig("dsssp_last_error", C.c_char_p)
_sig("dsssp_strerror", C.c_char_p, C.c_int)
_sig("dsssp_default_opts", None, C.POINTER(Opts))
_sig("dsssp_graph_create", C.c_int, C.c_int32, C.c_int64, _i32p, _i32p, _i32p, C.POINTER(Opts), C.POINTER(_P))
_sig("dsssp_graph_destroy", None, _P)
_sig("dsssp_graph_info", C.c_int, _P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
     C.POINTER(C.c_int64), C.POINTER(C.c_int32))
_sig("dsssp_tree_load", C.c_int, _P, _i32p, _i64p)
_sig("dsssp_tree_compute", C.c_int, _P, C.c_int32, C.POINTER(Stats))
_sig("dsssp_tree_compute_multi", C.c_int, _P, _i32p, C.c_int32, C.POINTER(Stats))
_sig("dsssp_forest_load", C.c_int, _P, _i32p, _i64p)
_sig("dsssp_tree_add_sources", C.c_int, _P, _i32p, C.c_int32, C.POINTER(Stats))
_sig("dsssp_graph_clear_range", C.c_int, _P, C.c_int32, C.c_int32)
_sig("dsssp_tree_read", C.c_int, _P, _P, _P)
_sig("dsssp_tree_read32", C.c_int, _P, _P, _P)
_sig("dsssp_tree_read32_async", C.c_int, _P, _P, _P)
_sig("dsssp_tree_read_wait", C.c_int, _P)
_sig("dsssp_tree_read_changed", C.c_int, _P, _P, _P, _P, C.c_int64, C.POINTER(C.c_int64))
_sig("dsssp_tree_validate", C.c_int, _P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int32))
_sig("dsssp_debug_set", C.c_int, _P, C.c_int32, C.c_int64)
DEBUG_SPIN_LIMIT = 1
DEBUG_STALL_US = 2


class ServerOpts(C.Structure):
    _fields_ = [
        ("memory_budget", C.c_int64),
        ("max_epoch_requests", C.c_int32),
        ("record", C.c_int32),
        ("compact_dead_frac", C.c_double),
        ("compact_spare_frac", C.c_double),
        ("reserve_vertices", C.c_int64),
        ("tune_cache", C.c_char_p),
    ]


class RequestInfo(C.Structure):
    _fields_ = [
        ("id", C.c_int64),
        ("tenant", C.c_int32),
        ("status", C.c_int32),
        ("epoch", C.c_int64),
        ("changes", C.c_int64),
        ("arrival_us", C.c_double),
        ("start_us", C.c_double),
        ("done_us", C.c_double),
        ("error", C.c_char * 96),
    ]


REFUSED = 1
W_RECOMPUTED = 2  # a batch recovered by recomputing the trees (a success code)
TENANT_WAITING, TENANT_ADMITTED, TENANT_REMOVED = 0, 1, 2
_PP = C.POINTER(C.c_void_p)
_sig("dsssp_tree_read_range", C.c_int, _P, C.c_int32, C.c_int32, _P, _P)
_sig("dsssp_pool_create", C.c_int, C.c_int32, _P, _P, _PP, _PP, _PP, C.POINTER(Opts), C.POINTER(_P))
_sig("dsssp_pool_destroy", None, _P)
_sig("dsssp_pool_create_reserved", C.c_int, C.c_int32, _P, _P, _PP, _PP, _PP, C.c_int64, C.POINTER(Opts),
     C.POINTER(_P))
_sig("dsssp_pool_add_graph", C.c_int, _P, C.c_int32, C.c_int64, _P, _P, _P, C.c_int32, C.POINTER(C.c_int32))
_sig("dsssp_pool_remove_graph", C.c_int, _P, C.c_int32)
_sig("dsssp_pool_graph_range", C.c_int, _P, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_int32))
_sig("dsssp_pool_capacity", C.c_int, _P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64))
_sig("dsssp_pool_graph", _P, _P)
_sig("dsssp_pool_offsets", C.c_int, _P, _P)
_sig("dsssp_pool_tree_compute", C.c_int, _P, _P, C.POINTER(Stats))
_sig("dsssp_pool_forest_load", C.c_int, _P, _PP, _PP)
_sig("dsssp_pool_union", C.c_int, _P, C.c_int32, _P, _PP, _P, _P, C.c_int64, C.POINTER(C.c_int64))
_sig("dsssp_pool_apply", C.c_int, _P, C.c_int32, _P, _PP, _P, C.POINTER(Stats))
_sig("dsssp_pool_tree_read", C.c_int, _P, C.c_int32, _P, _P)
_sig("dsssp_estimate_footprint", C.c_int64, C.c_int32, C.c_int64, C.c_int32, C.c_int32)
_sig("dsssp_default_server_opts", None, C.POINTER(ServerOpts))
_sig("dsssp_server_create", C.c_int, C.c_int32, _P, _P, _PP, _PP, _PP, _P, C.POINTER(ServerOpts), C.POINTER(Opts),
     C.POINTER(_P))
_sig("dsssp_server_destroy", None, _P)
_sig("dsssp_server_slot", C.c_int, _P, C.c_int32)
_sig("dsssp_server_tenant_state", C.c_int, _P, C.c_int32)
_sig("dsssp_server_add_tenant", C.c_int, _P, C.c_int32, C.c_int64, _P, _P, _P, C.c_int32, C.POINTER(C.c_int32))
_sig("dsssp_server_remove_tenant", C.c_int, _P, C.c_int32)
_sig("dsssp_server_recovered_epochs", C.c_int, _P, C.POINTER(C.c_int64))
_sig("dsssp_server_debug_set", C.c_int, _P, C.c_int32, C.c_int64)
_sig("dsssp_submit", C.c_int, _P, C.c_int32, _P, C.c_int64, C.POINTER(C.c_int64))
_sig("dsssp_submit_many", C.c_int, _P, C.c_int32, _P, _PP, _P, _P)
_sig("dsssp_poll", C.c_int, _P, C.POINTER(RequestInfo), C.c_int32, C.c_int32, C.POINTER(C.c_int32))
_sig("dsssp_server_drain", C.c_int, _P, C.c_int32)
_sig("dsssp_server_result", C.c_int, _P, C.c_int64, _P, _P)
_sig("dsssp_server_tree_read", C.c_int, _P, C.c_int32, _P, _P)
_sig("dsssp_server_info", C.c_int, _P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_double),
     C.POINTER(C.c_int64))
_sig("dsssp_server_pool", _P, _P)
_sig("dsssp_server_set_record", C.c_int, _P, C.c_int32)
_sig("dsssp_server_validate", C.c_int, _P, C.POINTER(C.c_int64), C.POINTER(C.c_int64))
_sig("dsssp_apply_batch", C.c_int, _P, _P, C.c_int64, _P, C.POINTER(Stats))
_sig("dsssp_apply_batch_async", C.c_int, _P, _P, C.c_int64, _P)
_sig("dsssp_apply_batch_host_async", C.c_int, _P, _P, C.c_int64, _P)
_sig("dsssp_batch_finish", C.c_int, _P, C.POINTER(Stats))
_sig("dsssp_graph_set_opts", C.c_int, _P, C.POINTER(Opts))
_sig("dsssp_graph_get_opts", C.c_int, _P, C.POINTER(Opts))
_sig("dsssp_graph_snapshot", C.c_int, _P)
_sig("dsssp_graph_restore", C.c_int, _P, _P)
_sig("dsssp_graph_compact", C.c_int, _P)
_sig("dsssp_graph_health", C.c_int, _P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
     C.POINTER(C.c_int64))
_sig("dsssp_host_alloc", _P, C.c_size_t)
_sig("dsssp_host_free", None, _P)
_sig("dsssp_launch_count", C.c_int64)
_sig("dsssp_free", None, _P)
_sig("dsssp_read_graph_file", C.c_int, C.c_char_p, C.c_int32, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P),
     C.POINTER(C.c_int64))
_sig("dsssp_read_changes_file", C.c_int, C.c_char_p, C.c_int32, C.POINTER(_P), C.POINTER(C.c_int64))
_sig("dsssp_read_sssp_file", C.c_int, C.c_char_p, C.c_int32, _i32p, _i64p, C.POINTER(C.c_int64))
_sig("dsssp_write_sssp_file", C.c_int, C.c_char_p, C.c_int32, _i32p, _i64p)
_sig("dsssp_gen_er", C.c_int, C.c_int32, C.c_int64, C.c_int32, C.c_int32, C.c_uint64, C.POINTER(_P),
     C.POINTER(_P), C.POINTER(_P))
_sig("dsssp_gen_rmat", C.c_int, C.c_int32, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32,
     C.c_uint64, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P))
_sig("dsssp_gen_grid", C.c_int, C.c_int32, C.c_int32, C.c_double, C.c_int64, C.c_int32, C.c_int32, C.c_uint64,
     C.POINTER(_P), C.POINTER(_P), C.POINTER(_P), C.POINTER(C.c_int64))
_sig("dsssp_gen_changes", C.c_int, C.c_int32, C.c_int64, _i32p, _i32p, _i32p, C.c_int64, C.c_int64, C.c_int32,
     C.c_int32, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32, C.c_uint64, C.POINTER(_P))
_sig("dsssp_max_degree_vertex", C.c_int32, C.c_int32, C.c_int64, _i32p, _i32p)
_sig("dsssp_gen_changes_ref", C.c_int, C.c_int32, C.c_int64, _i32p, _i32p, _i32p, C.c_int64, C.c_int32, C.c_int32,
     C.c_int32, C.c_uint64, C.POINTER(_P))
_sig("dsssp_write_changes_file", C.c_int, C.c_char_p, _P, C.c_int64)
_sig("dsssp_write_graph_binary", C.c_int, C.c_char_p, C.c_int32, C.c_int64, _i32p, _i32p, _i32p)
_sig("dsssp_read_graph_binary", C.c_int, C.c_char_p, C.c_int32, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P),
     C.POINTER(C.c_int64))
_sig("dsssp_write_sssp_binary", C.c_int, C.c_char_p, C.c_int32, _i32p, _i64p)
_sig("dsssp_read_sssp_binary", C.c_int, C.c_char_p, C.c_int32, _i32p, _i64p)
_sig("dsssp_sssp_noalloc", C.c_int, C.c_int32, C.c_int64, _P, _P, C.c_int32, _P, _P, _P)

_sig("dsssp_abi_sizes", C.c_int, C.POINTER(C.c_size_t), C.c_int32)


def abi_sizes() -> list[int]:
    """sizeof(dsssp_opts, dsssp_stats, dsssp_server_opts, dsssp_request_info,
    dsssp_tune_result) as the loaded library was built."""
    out = (C.c_size_t * 8)()
    k = _lib.dsssp_abi_sizes(out, 8)
    return [int(out[i]) for i in range(k)]


_built = abi_sizes()
_bound = [C.sizeof(Opts), C.sizeof(Stats), C.sizeof(ServerOpts), C.sizeof(RequestInfo)]
if _built[:4] != _bound:
    raise ImportError(f"{LIB_PATH}: built with struct sizes {_built[:4]}, this binding expects {_bound} "
                      "(rebuild the library: python -c 'import __graft_entry__ as g; g.build()')")

NOALLOC_MAX_VERTICES = 65536
NOALLOC_MAX_ENTRIES = 1 << 20

EXPORTED = [
    "dsssp_default_opts", "dsssp_graph_create", "dsssp_graph_destroy", "dsssp_graph_info", "dsssp_tree_load",
    "dsssp_tree_compute", "dsssp_tree_compute_multi", "dsssp_forest_load", "dsssp_tree_read", "dsssp_tree_read32", "dsssp_tree_read32_async", "dsssp_tree_read_wait", "dsssp_apply_batch", "dsssp_apply_batch_async", "dsssp_batch_finish",
    "dsssp_graph_set_opts", "dsssp_graph_get_opts", "dsssp_graph_snapshot", "dsssp_graph_restore", "dsssp_graph_compact", "dsssp_host_alloc", "dsssp_host_free",
    "dsssp_launch_count", "dsssp_last_error", "dsssp_strerror", "dsssp_free", "dsssp_read_graph_file",
    "dsssp_read_changes_file", "dsssp_read_sssp_file", "dsssp_write_sssp_file", "dsssp_gen_er", "dsssp_gen_rmat",
    "dsssp_gen_grid", "dsssp_gen_changes", "dsssp_max_degree_vertex", "dsssp_sssp_noalloc",
    "dsssp_gen_changes_ref", "dsssp_write_changes_file", "dsssp_write_graph_binary", "dsssp_read_graph_binary",
    "dsssp_write_sssp_binary", "dsssp_read_sssp_binary", "dsssp_graph_health", "dsssp_tree_read_changed",
    "dsssp_tree_validate", "dsssp_debug_set", "dsssp_tree_read_range",
    "dsssp_pool_create", "dsssp_pool_destroy", "dsssp_pool_graph", "dsssp_pool_offsets", "dsssp_pool_tree_compute",
    "dsssp_pool_forest_load", "dsssp_pool_union", "dsssp_pool_apply", "dsssp_pool_tree_read",
    "dsssp_estimate_footprint", "dsssp_default_server_opts", "dsssp_server_create", "dsssp_server_destroy",
    "dsssp_server_slot", "dsssp_submit", "dsssp_submit_many", "dsssp_poll", "dsssp_server_drain",
    "dsssp_server_result", "dsssp_server_tree_read", "dsssp_server_info", "dsssp_server_pool",
    "dsssp_server_set_record", "dsssp_server_validate", "dsssp_tree_add_sources", "dsssp_graph_clear_range",
    "dsssp_pool_create_reserved", "dsssp_pool_add_graph", "dsssp_pool_remove_graph", "dsssp_pool_graph_range",
    "dsssp_pool_capacity", "dsssp_server_tenant_state", "dsssp_server_add_tenant", "dsssp_server_remove_tenant",
    "dsssp_server_recovered_epochs", "dsssp_server_debug_set", "dsssp_apply_batch_host_async",
    "dsssp_autotune", "dsssp_autotune_lookup", "dsssp_tune_size_class", "dsssp_tune_candidates",
    "dsssp_abi_sizes",
]


def _check(rc: int, what: str) -> int:
    """Raises on a negative status; returns 0 or a positive success code (W_RECOMPUTED)."""
    if rc < 0:
        raise DsssspError(rc, what)
    return rc


def _take_i32(p: C.c_void_p, n: int) -> np.ndarray:
    if n == 0:
        _lib.dsssp_free(p)
        return np.zeros(0, np.int32)
    arr = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_int32)), shape=(n,)).copy()
    _lib.dsssp_free(p)
    return arr


def _take_changes(p: C.c_void_p, n: int) -> np.ndarray:
    if n == 0:
        _lib.dsssp_free(p)
        return np.zeros(0, CHANGE_DTYPE)
    buf = (C.c_char * (16 * n)).from_address(p.value)
    arr = np.frombuffer(bytes(buf), dtype=CHANGE_DTYPE).copy()
    _lib.dsssp_free(p)
    return arr


def default_opts(**kw) -> Opts:
    o = Opts()
    _lib.dsssp_default_opts(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError(f"unknown option {k}")
        setattr(o, k, v)
    return o


def make_changes(u, v, w, op) -> np.ndarray:
    ch = np.zeros(len(u), CHANGE_DTYPE)
    ch["u"], ch["v"], ch["w"], ch["op"] = u, v, w, op
    return ch


def launch_count() -> int:
    return int(_lib.dsssp_launch_count())


class Graph:
    """Device-resident graph + shortest-path tree (one GPU)."""

    def __init__(self, n: int, u, v, w, opts: Opts | None = None, **kw):
        u = np.ascontiguousarray(u, np.int32)
        v = np.ascontiguousarray(v, np.int32)
        w = np.ascontiguousarray(w, np.int32)
        if not (len(u) == len(v) == len(w)):
            raise ValueError("edge arrays differ in length")
        o = opts if opts is not None else default_opts(**kw)
        h = _P()
        _check(_lib.dsssp_graph_create(int(n), len(u), u, v, w, C.byref(o), C.byref(h)), "graph_create")
        self._h = h
        self.n = int(n)

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            _lib.dsssp_graph_destroy(self._h)
            self._h = _P()

    def __del__(self):
        self.close()  # dispatches to a subclass's close (a pool's graph is owned by the pool)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def info(self) -> dict:
        n, e, c, b = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        s = C.c_int32()
        _check(_lib.dsssp_graph_info(self._h, C.byref(n), C.byref(e), C.byref(c), C.byref(b), C.byref(s)), "info")
        return {"n": n.value, "entries": e.value, "capacity": c.value, "device_bytes": b.value, "source": s.value}

    def health(self) -> dict:
        """Live and tombstoned adjacency entries, used and total spare-region slots."""
        a, b, c, d = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        _check(_lib.dsssp_graph_health(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)), "health")
        return {"live": a.value, "dead": b.value, "spare_used": c.value, "spare_total": d.value}

    def tree_load(self, parent, dist) -> None:
        parent = np.ascontiguousarray(parent, np.int32)
        dist = np.ascontiguousarray(dist, np.int64)
        if len(parent) != self.n or len(dist) != self.n:
            raise ValueError("tree arrays must have n entries")
        _check(_lib.dsssp_tree_load(self._h, parent, dist), "tree_load")

    def tree_compute(self, src: int) -> Stats:
        st = Stats()
        _check(_lib.dsssp_tree_compute(self._h, int(src), C.byref(st)), "tree_compute")
        return st

    def tree_compute_multi(self, srcs) -> Stats:
        srcs = np.ascontiguousarray(srcs, np.int32)
        st = Stats()
        _check(_lib.dsssp_tree_compute_multi(self._h, srcs, len(srcs), C.byref(st)), "tree_compute_multi")
        return st

    def tree_add_sources(self, srcs) -> Stats:
        """New roots joined to the resident forest (relaxation from them; nothing recomputed)."""
        srcs = np.ascontiguousarray(srcs, np.int32)
        st = Stats()
        _check(_lib.dsssp_tree_add_sources(self._h, srcs, len(srcs), C.byref(st)), "tree_add_sources")
        return st

    def clear_range(self, first: int, count: int) -> None:
        """Removes every edge of ids [first, first + count) (closed under adjacency)."""
        _check(_lib.dsssp_graph_clear_range(self._h, int(first), int(count)), "clear_range")

    def forest_load(self, parent, dist) -> None:
        parent = np.ascontiguousarray(parent, np.int32)
        dist = np.ascontiguousarray(dist, np.int64)
        if len(parent) != self.n or len(dist) != self.n:
            raise ValueError("tree arrays must have n entries")
        _check(_lib.dsssp_forest_load(self._h, parent, dist), "forest_load")

    def tree_read(self, parent: np.ndarray | None = None, dist: np.ndarray | None = None):
        if parent is None:
            parent = np.empty(self.n, np.int32)
        if dist is None:
            dist = np.empty(self.n, np.int64)
        _check(_lib.dsssp_tree_read(self._h, parent.ctypes.data, dist.ctypes.data), "tree_read")
        return parent, dist

    def tree_read32(self, parent: np.ndarray | None = None, dist: np.ndarray | None = None):
        """(parent int32, dist uint32): the tree with 32-bit distances, UNREACHABLE32 where
        unreachable (8 bytes per vertex over the host link instead of 12)."""
        if parent is None:
            parent = np.empty(self.n, np.int32)
        if dist is None:
            dist = np.empty(self.n, np.uint32)
        _check(_lib.dsssp_tree_read32(self._h, parent.ctypes.data, dist.ctypes.data), "tree_read32")
        return parent, dist

    def tree_read32_async(self, parent_ptr: int | None, dist_ptr: int | None) -> None:
        """Starts copying the tree (int32 parents, uint32 distances) to host buffers of n
        entries at these addresses (pinned for an asynchronous copy); tree_read_wait() waits
        for it.  The next batch may be applied meanwhile."""
        _check(_lib.dsssp_tree_read32_async(self._h, parent_ptr, dist_ptr), "tree_read32_async")

    def tree_read_wait(self) -> None:
        _check(_lib.dsssp_tree_read_wait(self._h), "tree_read_wait")

    def debug_set(self, what: int, value: int) -> None:
        """Failure-detection test hooks (DEBUG_SPIN_LIMIT, DEBUG_STALL_US)."""
        _check(_lib.dsssp_debug_set(self._h, int(what), int(value)), "debug_set")

    def validate(self) -> dict:
        """Device-side certificate of the resident tree: {violations, roots, first_bad}."""
        bad, roots, first = C.c_int64(), C.c_int64(), C.c_int32()
        _check(_lib.dsssp_tree_validate(self._h, C.byref(bad), C.byref(roots), C.byref(first)), "tree_validate")
        return {"violations": bad.value, "roots": roots.value, "first_bad": first.value}

    def tree_read_changed(self, vertex: np.ndarray | None = None, parent: np.ndarray | None = None,
                          dist: np.ndarray | None = None):
        """(vertex, parent, dist) of every vertex the last batch may have changed (unordered);
        buffers of n entries may be passed in (pinned ones for fast copies)."""
        vertex = np.empty(self.n, np.int32) if vertex is None else vertex
        parent = np.empty(self.n, np.int32) if parent is None else parent
        dist = np.empty(self.n, np.int64) if dist is None else dist
        cnt = C.c_int64()
        _check(_lib.dsssp_tree_read_changed(self._h, vertex.ctypes.data, parent.ctypes.data, dist.ctypes.data,
                                            min(len(vertex), len(parent), len(dist)), C.byref(cnt)),
               "tree_read_changed")
        k = cnt.value
        return vertex[:k], parent[:k], dist[:k]

    def apply_batch(self, changes: np.ndarray, stream: int | None = None) -> Stats:
        changes = np.ascontiguousarray(changes, CHANGE_DTYPE)
        st = Stats()
        _check(_lib.dsssp_apply_batch(self._h, changes.ctypes.data, len(changes), stream, C.byref(st)),
               "apply_batch")
        return st

    def apply_batch_async(self, d_changes: int, k: int, stream: int | None = None) -> None:
        _check(_lib.dsssp_apply_batch_async(self._h, d_changes, int(k), stream), "apply_batch_async")

    def batch_finish(self) -> Stats:
        st = Stats()
        _check(_lib.dsssp_batch_finish(self._h, C.byref(st)), "batch_finish")
        return st

    def set_opts(self, opts: Opts) -> None:
        _check(_lib.dsssp_graph_set_opts(self._h, C.byref(opts)), "set_opts")

    def get_opts(self) -> Opts:
        o = Opts()
        _check(_lib.dsssp_graph_get_opts(self._h, C.byref(o)), "get_opts")
        return o

    def snapshot(self) -> None:
        _check(_lib.dsssp_graph_snapshot(self._h), "snapshot")

    def restore(self, stream: int | None = None) -> None:
        _check(_lib.dsssp_graph_restore(self._h, stream), "restore")

    def compact(self) -> None:
        _check(_lib.dsssp_graph_compact(self._h), "compact")


# ---- text formats ---------------------------------------------------------------------------

def read_graph(path: str, n: int):
    u, v, w, m = _P(), _P(), _P(), C.c_int64()
    _check(_lib.dsssp_read_graph_file(str(path).encode(), int(n), C.byref(u), C.byref(v), C.byref(w), C.byref(m)),
           "read_graph")
    return _take_i32(u, m.value), _take_i32(v, m.value), _take_i32(w, m.value)


def read_changes(path: str, n: int) -> np.ndarray:
    p, k = _P(), C.c_int64()
    _check(_lib.dsssp_read_changes_file(str(path).encode(), int(n), C.byref(p), C.byref(k)), "read_changes")
    return _take_changes(p, k.value)


def read_sssp(path: str, n: int):
    parent = np.empty(n, np.int32)
    dist = np.empty(n, np.int64)
    lossy = C.c_int64()
    _check(_lib.dsssp_read_sssp_file(str(path).encode(), int(n), parent, dist, C.byref(lossy)), "read_sssp")
    return parent, dist, lossy.value


def write_sssp(path: str, parent, dist) -> None:
    parent = np.ascontiguousarray(parent, np.int32)
    dist = np.ascontiguousarray(dist, np.int64)
    _check(_lib.dsssp_write_sssp_file(str(path).encode(), len(parent), parent, dist), "write_sssp")


def write_changes(path: str, changes: np.ndarray) -> None:
    """Change records in the reference generator's line format (createChangedEdges.cpp:104, 116)."""
    changes = np.ascontiguousarray(changes, CHANGE_DTYPE)
    _check(_lib.dsssp_write_changes_file(str(path).encode(), changes.ctypes.data if len(changes) else None,
                                         len(changes)), "write_changes")


def write_graph_binary(path: str, n: int, u, v, w) -> None:
    u = np.ascontiguousarray(u, np.int32)
    v = np.ascontiguousarray(v, np.int32)
    w = np.ascontiguousarray(w, np.int32)
    _check(_lib.dsssp_write_graph_binary(str(path).encode(), int(n), len(u), u, v, w), "write_graph_binary")


def read_graph_binary(path: str, n: int):
    u, v, w, m = _P(), _P(), _P(), C.c_int64()
    _check(_lib.dsssp_read_graph_binary(str(path).encode(), int(n), C.byref(u), C.byref(v), C.byref(w),
                                        C.byref(m)), "read_graph_binary")
    return _take_i32(u, m.value), _take_i32(v, m.value), _take_i32(w, m.value)


def write_sssp_binary(path: str, parent, dist) -> None:
    parent = np.ascontiguousarray(parent, np.int32)
    dist = np.ascontiguousarray(dist, np.int64)
    _check(_lib.dsssp_write_sssp_binary(str(path).encode(), len(parent), parent, dist), "write_sssp_binary")


def read_sssp_binary(path: str, n: int):
    parent = np.empty(n, np.int32)
    dist = np.empty(n, np.int64)
    _check(_lib.dsssp_read_sssp_binary(str(path).encode(), int(n), parent, dist), "read_sssp_binary")
    return parent, dist


# ---- generators -----------------------------------------------------------------------------

def gen_er(n: int, m: int, wlo: int = 1, whi: int = 100, seed: int = 0):
    u, v, w = _P(), _P(), _P()
    _check(_lib.dsssp_gen_er(n, m, wlo, whi, seed, C.byref(u), C.byref(v), C.byref(w)), "gen_er")
    return _take_i32(u, m), _take_i32(v, m), _take_i32(w, m)


def gen_rmat(scale: int, m: int, a=0.57, b=0.19, c=0.19, wlo: int = 1, whi: int = 100, seed: int = 0):
    u, v, w = _P(), _P(), _P()
    _check(_lib.dsssp_gen_rmat(scale, m, a, b, c, wlo, whi, seed, C.byref(u), C.byref(v), C.byref(w)), "gen_rmat")
    return _take_i32(u, m), _take_i32(v, m), _take_i32(w, m)


def gen_grid(rows: int, cols: int, remove_frac: float, n_diag: int, wlo: int = 1, whi: int = 1000, seed: int = 0):
    u, v, w, m = _P(), _P(), _P(), C.c_int64()
    _check(_lib.dsssp_gen_grid(rows, cols, remove_frac, n_diag, wlo, whi, seed, C.byref(u), C.byref(v), C.byref(w),
                               C.byref(m)), "gen_grid")
    return _take_i32(u, m.value), _take_i32(v, m.value), _take_i32(w, m.value)


def gen_changes(n: int, u, v, w, n_ins: int, n_del: int, kind: int = INS_UNIFORM, scale: int = 0,
                p0: float = 0.0, p1: float = 0.0, p2: float = 0.0, wlo: int = 1, whi: int = 100,
                seed: int = 0) -> np.ndarray:
    u = np.ascontiguousarray(u, np.int32)
    v = np.ascontiguousarray(v, np.int32)
    w = np.ascontiguousarray(w, np.int32)
    p = _P()
    _check(_lib.dsssp_gen_changes(n, len(u), u, v, w, n_ins, n_del, kind, scale, p0, p1, p2, wlo, whi, seed,
                                  C.byref(p)), "gen_changes")
    return _take_changes(p, n_ins + n_del)


def gen_changes_ref(n: int, u, v, w, num_changes: int, ins_pct: int, wlo: int = 0, whi: int = 99,
                    seed: int = 0) -> np.ndarray:
    """The reference generator's sampling (createChangedEdges.cpp:75-122), seeded: coin-flip
    interleaving, insertions of any pair u<v with w in [wlo, whi] (default [0, 99] as the
    reference), deletions drawn from the edge list with replacement."""
    u = np.ascontiguousarray(u, np.int32)
    v = np.ascontiguousarray(v, np.int32)
    w = np.ascontiguousarray(w, np.int32)
    p = _P()
    _check(_lib.dsssp_gen_changes_ref(n, len(u), u, v, w, num_changes, ins_pct, wlo, whi, seed, C.byref(p)),
           "gen_changes_ref")
    return _take_changes(p, num_changes)


def max_degree_vertex(n: int, u, v) -> int:
    u = np.ascontiguousarray(u, np.int32)
    v = np.ascontiguousarray(v, np.int32)
    return int(_lib.dsssp_max_degree_vertex(n, len(u), u, v))


def sssp_noalloc(n: int, nnz: int, d_row_off: int, d_adj: int, src: int, d_parent: int, d_dist: int,
                 stream: int | None = None) -> None:
    """Shortest-path tree of a CSR graph in caller device memory (raw device addresses);
    the engine allocates nothing for it (see dsssp_sssp_noalloc in include/dsssp.h)."""
    _check(_lib.dsssp_sssp_noalloc(int(n), int(nnz), d_row_off, d_adj, int(src), d_parent, d_dist, stream),
           "sssp_noalloc")
