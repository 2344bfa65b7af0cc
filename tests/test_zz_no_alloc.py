"""dsssp_sssp_noalloc: the shortest-path tree for callers that cannot allocate device memory
where they call the engine (an enqueue callback of a runtime that owns the memory budget, a
pipeline that reserved all device memory up front).  The test owns the device buffers (via
torch) and calls the entry point through the C ABI twice in a row -- the second call on a
different graph and source, so it also covers a work space left over from the previous call
-- comparing each result with the allocating path (dsssp_graph_create + dsssp_tree_compute):
distances bit-exact, the same unreachable set, and parents forming a valid shortest-path
tree.  This file is collected last on purpose."""
import numpy as np
import pytest

import dynamicssspv2_gb300 as D
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def _run_noalloc(torch, n, csr, src):
    adj = np.ascontiguousarray(np.stack([csr.col, csr.wt], axis=1).astype(np.int32))
    d_off = torch.from_numpy(csr.off.astype(np.int64)).cuda()
    d_adj = torch.from_numpy(adj.reshape(-1)).cuda()
    d_par = torch.full((n,), 7, dtype=torch.int32, device="cuda")
    d_dist = torch.full((n,), 7, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    D.sssp_noalloc(n, len(csr.col), d_off.data_ptr(), d_adj.data_ptr(), src, d_par.data_ptr(), d_dist.data_ptr())
    return d_par.cpu().numpy(), d_dist.cpu().numpy()


def test_noalloc_matches_allocating_path_twice():
    torch = pytest.importorskip("torch")
    cases = [(5000, 20000, 1, 0), (30000, 150000, 2, 17)]
    for n, m, seed, src in cases:
        u, v, w = D.gen_er(n, m, 1, 100, seed)
        csr = O.csr(n, u, v, w)
        assert len(csr.col) <= D.NOALLOC_MAX_ENTRIES and n <= D.NOALLOC_MAX_VERTICES
        par, dist = _run_noalloc(torch, n, csr, src)
        with D.Graph(n, u, v, w) as g:
            g.tree_compute(src)
            ref_par, ref_dist = g.tree_read()
        assert np.array_equal(dist, ref_dist)
        assert np.array_equal(par == -1, ref_par == -1)
        assert par[src] == src and dist[src] == 0
        # weights are >= 1, so the packed minimum's tie rule (least parent id among the tight
        # neighbours) makes the parents deterministic: both paths give the same tree
        assert np.array_equal(par, ref_par)
        assert O.validate(n, csr, src, dist, par) == 0


def test_noalloc_refuses_malformed_csr_then_recovers():
    """Each malformed CSR stays inside off[0..n] and adj[0..nnz) (what the set-up kernel reads)
    and must give DSSSP_E_INVAL; a valid call right after must still match the allocating
    path, so a refused call leaves nothing behind in the shared work space."""
    torch = pytest.importorskip("torch")
    n, m, src = 3000, 12000, 5
    u, v, w = D.gen_er(n, m, 1, 100, 9)
    csr = O.csr(n, u, v, w)
    adj = np.ascontiguousarray(np.stack([csr.col, csr.wt], axis=1).astype(np.int32))
    off = csr.off.astype(np.int64)
    bad = []
    o = off.copy()
    o[n] = len(csr.col) - 1  # last offset is not nnz
    bad.append(("last offset", o, adj))
    o = off.copy()
    o[n // 2] = o[n // 2 + 1] + 1  # offsets go down
    bad.append(("non-monotone offsets", o, adj))
    a = adj.copy()
    a[len(a) // 3, 0] = n  # a column equal to n
    bad.append(("column n", off, a))
    a = adj.copy()
    a[len(a) // 2, 1] = -1  # a negative weight
    bad.append(("negative weight", off, a))
    d_par = torch.zeros(n, dtype=torch.int32, device="cuda")
    d_dist = torch.zeros(n, dtype=torch.int64, device="cuda")
    for what, o, a in bad:
        d_off = torch.from_numpy(o).cuda()
        d_adj = torch.from_numpy(a.reshape(-1)).cuda()
        with pytest.raises(D.DsssspError) as e:
            D.sssp_noalloc(n, len(a), d_off.data_ptr(), d_adj.data_ptr(), src, d_par.data_ptr(), d_dist.data_ptr())
        assert e.value.code == D.E_INVAL, what
    par, dist = _run_noalloc(torch, n, csr, src)
    with D.Graph(n, u, v, w) as g:
        g.tree_compute(src)
        ref_par, ref_dist = g.tree_read()
    assert np.array_equal(dist, ref_dist) and np.array_equal(par, ref_par)


def test_noalloc_rejects_sizes_beyond_the_limit():
    torch = pytest.importorskip("torch")
    n = D.NOALLOC_MAX_VERTICES + 1
    d_off = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    d_out = torch.zeros(n, dtype=torch.int64, device="cuda")
    with pytest.raises(D.DsssspError) as e:
        D.sssp_noalloc(n, 0, d_off.data_ptr(), 0, 0, d_out.data_ptr(), d_out.data_ptr())
    assert e.value.code == D.E_INVAL
    with pytest.raises(D.DsssspError) as e:
        D.sssp_noalloc(10, D.NOALLOC_MAX_ENTRIES + 1, d_off.data_ptr(), d_out.data_ptr(), 0, d_out.data_ptr(),
                       d_out.data_ptr())
    assert e.value.code == D.E_INVAL
