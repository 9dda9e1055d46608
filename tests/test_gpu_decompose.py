"""Device-resident decomposition, k-truss search and triangle count through
the C ABI, against the reference's golden outputs and the oracle."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests import _golden as GD
from tdtdecomposition_gb300 import CSRCOO, generators as G, truss as T
from tdtdecomposition_gb300._lib import TdtError

pytestmark = pytest.mark.gpu
CASES = GD.names()


def graph_of(rows, cols, rp):
    return CSRCOO(columns=torch.as_tensor(cols, dtype=torch.int32).cuda(),
                  row_ptr=torch.as_tensor(np.asarray(rp), dtype=torch.int64).cuda(),
                  rows=torch.as_tensor(rows, dtype=torch.int32).cuda())


@pytest.mark.parametrize("name", CASES)
def test_decompose_matches_reference_peel_order(name):
    d = GD.load(name)
    g = graph_of(d["ref_rows"], d["ref_cols"], d["ref_rp"])
    res = T.truss_decompose(g)
    assert res.kmax == int(d["sg_kmax2"]) == int(d["sg_kmax1"])
    assert np.array_equal(res.e_truss.cpu().numpy(), d["sg_e_truss2"])
    assert np.array_equal(res.e_truss.cpu().numpy(), d["sg_e_truss1"])
    assert np.array_equal(res.ptr_truss.cpu().numpy(), d["sg_ptr_truss2"])
    E = d["ref_cols"].shape[0]
    assert np.array_equal(res.truss.cpu().numpy(), GD.truss_from_levels(d["sg_e_truss2"], d["sg_ptr_truss2"], E))
    assert res.triangles == int(d["ref_support"].sum()) // 3


@pytest.mark.parametrize("name", CASES)
def test_decompose_without_rows(name):
    d = GD.load(name)
    g = graph_of(d["ref_rows"], d["ref_cols"], d["ref_rp"])
    g.rows = None
    res = T.truss_decompose(g)
    assert np.array_equal(res.e_truss.cpu().numpy(), d["sg_e_truss2"])


@pytest.mark.parametrize("name", CASES)
def test_ktruss_search_matches_reference(name):
    d = GD.load(name)
    g = graph_of(d["ref_rows"], d["ref_cols"], d["ref_rp"])
    truss = GD.truss_from_levels(d["sg_e_truss2"], d["sg_ptr_truss2"], d["ref_cols"].shape[0])
    for k in list(d["kt_ks"]) + [1, 2]:
        m = T.ktruss_search(g, int(k)).cpu().numpy()
        assert np.array_equal(m, truss >= k), k
        if ("kt_rows_k%d" % k) in d:
            got = GD.edge_set(d["ref_rows"][m], d["ref_cols"][m])
            assert got == GD.edge_set(d["kt_rows_k%d" % k], d["kt_cols_k%d" % k])


@pytest.mark.parametrize("name", CASES)
def test_triangle_count(name):
    d = GD.load(name)
    g = graph_of(d["ref_rows"], d["ref_cols"], d["ref_rp"])
    t, sup = T.triangle_count(g, return_support=True)
    assert t == int(d["ref_support"].sum()) // 3
    assert np.array_equal(sup.cpu().numpy(), d["ref_support"])


def _oracle_check(pairs, n_cut=2):
    rows, cols, rp, verts = O.preprocess(pairs, stable=True)
    V = len(verts)
    kmax, et, pt, truss = O.k_truss(rows, cols, O.tiling_row_ptr(rows, cols, V, n_cut), V, n_cut)
    res = T.truss_decompose(graph_of(rows, cols, rp))
    assert res.kmax == kmax
    assert np.array_equal(res.ptr_truss.cpu().numpy(), pt)
    assert np.array_equal(res.e_truss.cpu().numpy(), et)
    assert np.array_equal(res.truss.cpu().numpy(), truss)
    return res


@pytest.mark.parametrize("scale", [12, 14])
def test_decompose_rmat_vs_oracle(scale):
    s, d = G.rmat_edges(scale, 16 << scale, seed=11)
    _oracle_check(np.stack([s, d], 1))


def test_decompose_ba_vs_oracle():
    s, d = G.ba_edges(20000, 12, seed=1234)
    _oracle_check(np.stack([s, d], 1))


def test_decompose_chung_lu_vs_oracle():
    s, d = G.chung_lu_edges(1 << 14, gamma=2.1, mean_degree=20, max_degree=2000, seed=2)
    _oracle_check(np.stack([s, d], 1))


def test_empty_graph():
    g = graph_of(np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(5, np.int64))
    res = T.truss_decompose(g)
    assert res.kmax == 2 and res.e_truss.numel() == 0 and res.ptr_truss.cpu().tolist() == [0]


def test_triangle_free_graph():
    # a star: the reference's loop never terminates here; this returns kmax 2
    pairs = np.array([[0, i] for i in range(1, 50)], np.int32)
    rows, cols, rp, verts = O.preprocess(pairs)
    res = T.truss_decompose(graph_of(rows, cols, rp))
    assert res.kmax == 2 and res.triangles == 0
    assert res.ptr_truss.cpu().tolist() == [0] and res.e_truss.numel() == 0
    assert np.all(res.truss.cpu().numpy() == 2)


def test_single_triangle_and_clique():
    for k in (3, 4, 12, 40):
        pairs = np.array([[a, b] for a in range(k) for b in range(a + 1, k)], np.int32)
        rows, cols, rp, verts = O.preprocess(pairs)
        res = T.truss_decompose(graph_of(rows, cols, rp))
        assert res.kmax == k
        assert np.all(res.truss.cpu().numpy() == k)
        assert res.triangles == k * (k - 1) * (k - 2) // 6


def test_rejects_unoriented_graph():
    rows = np.array([0, 2], np.int32)
    cols = np.array([1, 1], np.int32)  # edge 2 -> 1 is not low -> high
    rp = np.array([0, 1, 1, 2], np.int64)
    with pytest.raises(TdtError):
        T.truss_decompose(graph_of(rows, cols, rp))


def test_repeatable_and_workspace_reuse():
    s, d = G.rmat_edges(13, 16 << 13, seed=21)
    rows, cols, rp, verts = O.preprocess(np.stack([s, d], 1))
    g = graph_of(rows, cols, rp)
    ws = T.Workspace()
    a = T.truss_decompose(g, workspace=ws)
    b = T.truss_decompose(g, workspace=ws)
    assert torch.equal(a.truss, b.truss) and torch.equal(a.e_truss, b.e_truss)
