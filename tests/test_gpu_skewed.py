"""The skewed single-graph workload (Chung-Lu power law, exponent 2.1, mean
degree 40, degree cap 2^20): the device generator against the host one, and
at a size the oracle finishes in seconds, the path the workload runs —
GPU preprocessing, triangle count, full decomposition and k-truss search at
k in {3, 8, kmax/2, kmax} — against the oracle."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tdtdecomposition_gb300 import generators as G, truss as T
from tdtdecomposition_gb300.preprocess import preprocess_edges

pytestmark = pytest.mark.gpu


def test_device_generator_equals_host():
    n = 1 << 16
    s, d = G.chung_lu_edges(n, seed=2)
    sd, dd = G.chung_lu_edges_device(n, seed=2)
    assert np.array_equal(sd.cpu().numpy(), s) and np.array_equal(dd.cpu().numpy(), d)


def test_skewed_path_vs_oracle():
    n = 1 << 13
    s, d = G.chung_lu_edges(n, seed=2)
    sd, dd = G.chung_lu_edges_device(n, seed=2)
    g, verts = preprocess_edges(sd, dd)
    rows, cols, rp, v = O.preprocess(np.stack([s, d], 1), stable=True)
    assert np.array_equal(g.columns.cpu().numpy(), cols) and np.array_equal(g.rows.cpu().numpy(), rows)
    V = len(v)
    kmax, et, pt, truss = O.k_truss(rows, cols, O.tiling_row_ptr(rows, cols, V, 2), V, 2)
    sup = O.support(rows, cols, rp.astype(np.int32), 1)
    t, sup_d = T.triangle_count(g, return_support=True)
    assert t == int(sup.sum()) // 3 and np.array_equal(sup_d.cpu().numpy(), sup)
    for lists in (True, False):
        res = T.truss_decompose(g, lists=lists)
        assert res.listed == lists
        assert res.kmax == kmax and np.array_equal(res.truss.cpu().numpy(), truss)
        assert np.array_equal(res.e_truss.cpu().numpy(), et) and np.array_equal(res.ptr_truss.cpu().numpy(), pt)
        for k in sorted({3, 8, kmax // 2, kmax}):
            m = T.ktruss_search(g, k, lists=lists).cpu().numpy()
            assert np.array_equal(m, truss >= k), (lists, k)
