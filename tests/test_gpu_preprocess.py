"""Device preprocessing (tdt_preprocess) against the oracle's restatement of
Graph.read_edgelist + CSRCOO.edge_list_to_Graph with the (degree, id) rank;
the device R-MAT generator against the host one."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests import _golden as GD
from tdtdecomposition_gb300 import generators as G
from tdtdecomposition_gb300._lib import TdtError
from tdtdecomposition_gb300.preprocess import preprocess_edges

pytestmark = pytest.mark.gpu


def _check(pairs):
    pairs = np.asarray(pairs, np.int32).reshape(-1, 2)
    rows, cols, rp, verts = O.preprocess(pairs, stable=True)
    g, v = preprocess_edges(torch.as_tensor(pairs[:, 0]).cuda(), torch.as_tensor(pairs[:, 1]).cuda())
    assert np.array_equal(g.rows.cpu().numpy(), rows)
    assert np.array_equal(g.columns.cpu().numpy(), cols)
    assert np.array_equal(g.row_ptr.cpu().numpy(), rp.astype(np.int64))
    assert np.array_equal(v.cpu().numpy(), verts.astype(np.int32))


@pytest.mark.parametrize("name", GD.names())
def test_preprocess_golden_inputs(name):
    _check(GD.load(name)["pairs"])


def test_preprocess_self_loops_duplicates_and_gaps():
    pairs = np.array([[5, 5], [5, 9], [9, 5], [9, 5], [100, 9], [7, 7], [100, 5], [3, 100]], np.int32)
    _check(pairs)


def test_preprocess_rmat_and_chung_lu():
    _check(np.stack(G.rmat_edges(14, 16 << 14, seed=3), 1))
    _check(np.stack(G.chung_lu_edges(20000, mean_degree=12, max_degree=3000, seed=4), 1))


def test_preprocess_empty_and_invalid():
    z = torch.zeros(0, dtype=torch.int32, device="cuda")
    g, v = preprocess_edges(z, z)
    assert g.num_edges == 0 and v.numel() == 0
    with pytest.raises(TdtError):
        preprocess_edges(torch.tensor([0, 5], dtype=torch.int32, device="cuda"),
                         torch.tensor([1, 2], dtype=torch.int32, device="cuda"), num_ids=4)


@pytest.mark.parametrize("scale", [8, 16])
def test_device_rmat_matches_host(scale):
    s_h, d_h = G.rmat_edges(scale, 16 << scale, seed=1)
    s_d, d_d = G.rmat_edges_device(scale, 16 << scale, seed=1)
    assert np.array_equal(s_d.cpu().numpy(), s_h) and np.array_equal(d_d.cpu().numpy(), d_h)
