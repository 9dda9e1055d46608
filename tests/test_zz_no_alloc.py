"""tdt_triangle_count_noalloc: the triangle count for callers that cannot
allocate device memory (another component owns the allocator, or the path
must not stall on cudaMalloc).  Checked through the C ABI against the
workspace-based tdt_triangle_count on two calls in a row, so the second call
also shows that the shared static scratch left by the first one does not leak
into its result.  Collected last (file name) so that a run stopping at the
first failure has run every other test first."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests import _golden as GD
from tdtdecomposition_gb300 import _lib, generators as G

pytestmark = pytest.mark.gpu


def _graphs():
    """(rows, cols, row_ptr, expected support or None): the golden R-MAT
    scale-10 graph with the reference's own support, a scale-13 R-MAT graph,
    and the size limit's corner: 2^18 edges over about 227 K vertices."""
    d = GD.load("rmat_s10")
    yield d["ref_rows"], d["ref_cols"], d["ref_rp"], d["ref_support"]
    s, t = G.rmat_edges(13, 16 << 13, seed=5)
    rows, cols, rp, verts = O.preprocess(np.stack([s, t], 1))
    yield rows, cols, rp, None
    s, t = G.er_edges(1 << 18, 1 << 18, seed=3)
    rows, cols, rp, verts = O.preprocess(np.stack([s, t], 1))
    assert len(cols) == 1 << 18 and len(verts) > 200000
    yield rows, cols, rp, None


def _count_with_workspace(L, cols, rp, stream):
    V, E = rp.numel() - 1, cols.numel()
    ws = torch.empty(L.tdt_decompose_workspace_bytes(V, E), dtype=torch.uint8, device="cuda")
    sup = torch.full((E,), -7, dtype=torch.int32, device="cuda")
    stats = torch.zeros(8, dtype=torch.int64, device="cuda")
    rc = L.tdt_triangle_count(cols.data_ptr(), rp.data_ptr(), V, E, sup.data_ptr(), stats.data_ptr(),
                              ws.data_ptr(), ws.numel(), stream)
    assert rc == 0, L.tdt_last_error()
    torch.cuda.synchronize()
    return sup.cpu(), stats.cpu()


def test_noalloc_matches_workspace_entry_point_twice():
    L = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    for rows, cols_np, rp_np, golden in _graphs():
        cols = torch.as_tensor(cols_np, dtype=torch.int32).cuda()
        rp = torch.as_tensor(np.asarray(rp_np), dtype=torch.int64).cuda()
        V, E = rp.numel() - 1, cols.numel()
        ref_sup, ref_stats = _count_with_workspace(L, cols, rp, stream)
        assert int(ref_stats[0]) == 0
        if golden is not None:
            assert np.array_equal(ref_sup.numpy(), golden)
        for _ in range(2):
            sup = torch.full((E,), -7, dtype=torch.int32, device="cuda")
            stats = torch.full((8,), -1, dtype=torch.int64, device="cuda")
            rc = L.tdt_triangle_count_noalloc(cols.data_ptr(), rp.data_ptr(), V, E, sup.data_ptr(),
                                              stats.data_ptr(), stream)
            assert rc == 0, L.tdt_last_error()
            torch.cuda.synchronize()
            st = stats.cpu()
            assert int(st[0]) == 0
            assert int(st[4]) == int(ref_stats[4])  # triangles
            assert torch.equal(sup.cpu(), ref_sup)


def test_noalloc_rejects_graphs_beyond_its_limit():
    L = _lib.load()
    rc = L.tdt_triangle_count_noalloc(None, None, 10, (1 << 18) + 1, None, None, None)
    assert rc == 1  # TDT_ERR_INVALID, nothing launched
    assert b"at most" in L.tdt_last_error()
