"""The large graphs pinned to the oracle: the GPU decomposition of the
benchmark's R-MAT scale-22 graph and of Chung-Lu 2^18 / 2^20 graphs must
reproduce, bit for bit, the oracle's per-edge support, truss numbers, e_truss
and ptr_truss (SHA-256 digests in tests/golden/fullsize_digests.json, made by
tests/golden/make_fullsize_digests.py from the oracle's restatement of
demo_truss/singlegpu_truss.py:67-158).  The graph is generated and
preprocessed on the device; the digests of its columns and row_ptr show it is
the CSR the oracle ran on.  Both peels are checked: over per-edge triangle
lists and by search in the adjacency."""
import hashlib
import json
import os

import numpy as np
import pytest
import torch

from tdtdecomposition_gb300 import generators as G, truss as T
from tdtdecomposition_gb300.preprocess import preprocess_edges

pytestmark = pytest.mark.gpu

DIGESTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fullsize_digests.json")


def _cases():
    with open(DIGESTS) as f:
        return json.load(f)


def _sha(t, dtype):
    a = np.ascontiguousarray(t.cpu().numpy(), dtype=np.dtype(dtype).newbyteorder("<"))
    return hashlib.sha256(a.tobytes()).hexdigest()


def _graph(p):
    if p["kind"] == "rmat":
        src, dst = G.rmat_edges_device(p["scale"], p["edge_factor"] << p["scale"], seed=p["seed"])
    else:
        src, dst = G.chung_lu_edges_device(1 << p["log2n"], p["gamma"], p["mean_degree"], p["max_degree"],
                                           seed=p["seed"])
    g, _ = preprocess_edges(src, dst)
    return g


@pytest.mark.parametrize("name", ["chung_lu_18", "chung_lu_20", "rmat_s22"])
def test_decomposition_matches_oracle_digests(name):
    cases = _cases()
    if name not in cases:
        pytest.skip("no digests recorded for %s" % name)
    ref = cases[name]
    g = _graph(ref["params"])
    V, E = g.row_ptr.shape[0] - 1, g.columns.shape[0]
    assert (V, E) == (ref["V"], ref["E"])
    assert _sha(g.columns, np.int32) == ref["sha256"]["columns"]
    assert _sha(g.row_ptr, np.int64) == ref["sha256"]["row_ptr"]
    ws = T.Workspace()
    tri, sup = T.triangle_count(g, workspace=ws, return_support=True)
    assert tri == ref["triangles"]
    assert _sha(sup, np.int32) == ref["sha256"]["support"]
    del sup
    for lists in (True, False):
        res = T.truss_decompose(g, workspace=ws, lists=lists)
        assert res.listed == lists
        assert (res.kmax, res.triangles) == (ref["kmax"], ref["triangles"]), lists
        assert (res.e_truss.shape[0], res.ptr_truss.shape[0]) == (ref["n_etruss"], ref["n_ptr"]), lists
        assert _sha(res.truss, np.int32) == ref["sha256"]["truss"], lists
        assert _sha(res.e_truss, np.int32) == ref["sha256"]["e_truss"], lists
        assert _sha(res.ptr_truss, np.int32) == ref["sha256"]["ptr_truss"], lists
        del res
    del ws, g
    torch.cuda.empty_cache()
