"""Failure detection without a GPU fault: every device wait has a limit, and a
wait that runs out comes back as an error status while the context stays
usable.  The waits are made to run out on purpose here (a barrier one block
never reaches; a peel deadline shorter than the run), never by a fault."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tdtdecomposition_gb300 import CSRCOO, _lib, generators as G, truss as T
from tdtdecomposition_gb300._lib import TdtError

pytestmark = pytest.mark.gpu
TIMEOUT = 4  # TDT_ERR_TIMEOUT


def _graph(scale, seed):
    s, d = G.rmat_edges(scale, 16 << scale, seed=seed)
    pairs = np.stack([s, d], 1)
    rows, cols, rp, verts = O.preprocess(pairs)
    g = CSRCOO(columns=torch.as_tensor(cols, dtype=torch.int32).cuda(),
               row_ptr=torch.as_tensor(rp, dtype=torch.int64).cuda(),
               rows=torch.as_tensor(rows, dtype=torch.int32).cuda())
    return g, pairs


def test_grid_barrier_wait_runs_out_with_status():
    L = _lib.load()
    ws = torch.zeros(4096, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert L.tdt_test_barrier_timeout(ws.data_ptr(), 50_000_000, stream) == TIMEOUT
    # limits outside [1 ms, 2 s] are refused on the host
    assert L.tdt_test_barrier_timeout(ws.data_ptr(), 10, stream) == 1
    # the context is still usable
    g, _ = _graph(10, 4)
    assert T.triangle_count(g) > 0


def test_peel_deadline_stops_the_run_and_the_next_run_is_exact():
    L = _lib.load()
    g, pairs = _graph(14, 6)
    L.tdt_set_peel_deadline_ns(1)
    try:
        with pytest.raises(TdtError) as ei:
            T.truss_decompose(g)
        assert ei.value.status == TIMEOUT
    finally:
        L.tdt_set_peel_deadline_ns(0)
    rows, cols, rp, verts = O.preprocess(pairs, stable=True)
    kmax, et, pt, truss = O.k_truss(rows, cols, O.tiling_row_ptr(rows, cols, len(verts), 2), len(verts), 2)
    res = T.truss_decompose(g)
    assert res.kmax == kmax
    assert np.array_equal(res.truss.cpu().numpy(), truss)
