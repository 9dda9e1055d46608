"""The benchmark's graph at full size: R-MAT scale 22, edge factor 16
((a, b, c, d) = (.57, .19, .19, .05), seed 1; V = 2,396,037, E = 64,155,377,
2.11 G triangles).  The oracle needs minutes here, so the decomposition is
checked through properties that hold at any size:

* the support of every edge is the same from the whole-path kernel and from
  the drop-in `segment_isin2` operator, and sums to 3 T;
* e_truss is a permutation of the edges that lie in a triangle (the others
  have truss number 2), and ptr_truss cuts it into levels: entries
  ptr_truss[i] .. ptr_truss[i+1] are the edges of truss number i + 3;
* the peel without lists (triangles found by binary search in the adjacency)
  gives the same three outputs as the peel over per-edge lists;
* for k in {3, 8, kmax/2, kmax}: every edge of H_k = {e : truss(e) >= k} lies
  in at least k - 2 triangles of H_k (H_k is a k-truss), and the fixed-level
  peel of the whole graph at k (ktruss_search/ktruss_cuda.py:383-463) keeps
  exactly H_k (no larger k-truss exists); H_{kmax+1} is empty;
* a second run is bit-identical.
"""
import pytest
import torch

from tdtdecomposition_gb300 import CSRCOO, generators as G, truss as T, trusstensor as tt
from tdtdecomposition_gb300.preprocess import preprocess_edges

pytestmark = pytest.mark.gpu

SCALE, EDGE_FACTOR, SEED = 22, 16, 1


@pytest.fixture(scope="module")
def big():
    src, dst = G.rmat_edges_device(SCALE, EDGE_FACTOR << SCALE, seed=SEED)
    g, _ = preprocess_edges(src, dst)
    del src, dst
    ws = T.Workspace()
    res = T.truss_decompose(g, workspace=ws, lists=True)
    assert res.listed
    yield g, ws, res
    del ws
    torch.cuda.empty_cache()


def test_fullsize_shape(big):
    g, _, res = big
    assert (g.row_ptr.shape[0] - 1, g.columns.shape[0]) == (2396037, 64155377)
    assert (res.kmax, res.triangles, res.rounds) == (546, 2111711682, 4034)


def test_fullsize_support_two_paths(big):
    g, ws, res = big
    tri, sup = T.triangle_count(g, workspace=ws, return_support=True)
    assert tri == res.triangles
    assert int(sup.sum(dtype=torch.int64)) == 3 * tri
    out = torch.zeros_like(sup)
    tt.segment_isin2(g.rows, g.columns, g.row_ptr.to(torch.int32), out)
    assert torch.equal(out, sup)


def test_fullsize_peel_order(big):
    g, ws, res = big
    et, pt, truss = res.e_truss.long(), res.ptr_truss.long(), res.truss
    _, sup = T.triangle_count(g, workspace=ws, return_support=True)
    assert torch.equal(truss == 2, sup == 0)
    in_tri = torch.nonzero(sup > 0).squeeze(1)
    assert torch.equal(torch.sort(et).values, in_tri)
    assert pt.shape[0] == res.kmax - 1
    assert int(pt[0]) == 0 and int(pt[-1]) == et.shape[0] and bool((pt[1:] >= pt[:-1]).all())
    lvl = torch.repeat_interleave(torch.arange(pt.shape[0] - 1, device=et.device), pt[1:] - pt[:-1])
    assert torch.equal(truss[et], (lvl + 3).to(torch.int32))
    assert int(truss.min()) >= 2 and int(truss.max()) == res.kmax


def test_fullsize_search_peel_agrees(big):
    g, ws, res = big
    s = T.truss_decompose(g, workspace=ws, lists=False)
    assert not s.listed
    assert torch.equal(s.truss, res.truss)
    assert torch.equal(s.e_truss, res.e_truss) and torch.equal(s.ptr_truss, res.ptr_truss)


def _sub_csr(g, keep):
    rows, cols = g.rows[keep], g.columns[keep]
    V = g.row_ptr.shape[0] - 1
    rp = torch.zeros(V + 1, dtype=torch.int64, device=cols.device)
    rp[1:] = torch.cumsum(torch.bincount(rows.long(), minlength=V), 0)
    return CSRCOO(columns=cols.contiguous(), row_ptr=rp, rows=rows.contiguous())


def test_fullsize_levels_are_maximal_trusses(big):
    g, ws, res = big
    for k in (3, 8, res.kmax // 2, res.kmax):
        keep = res.truss >= k
        h = _sub_csr(g, keep)
        _, sup = T.triangle_count(h, workspace=ws, return_support=True)
        assert int(sup.min()) >= k - 2, k
        assert torch.equal(T.ktruss_search(g, k, workspace=ws), keep), k
    assert not bool(T.ktruss_search(g, res.kmax + 1, workspace=ws).any())


def test_fullsize_repeatable(big):
    g, ws, res = big
    again = T.truss_decompose(g, workspace=ws, lists=True)
    assert torch.equal(again.truss, res.truss)
    assert torch.equal(again.e_truss, res.e_truss) and torch.equal(again.ptr_truss, res.ptr_truss)
