"""Batched decomposition (disjoint union in one device-resident run) against
each graph decomposed alone and against the oracle; device preprocessing with
vertex groups; the autotuner."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tdtdecomposition_gb300 import autotune, batch as B, generators as G, truss as T, workloads as W
from tdtdecomposition_gb300.graph import CSRCOO
from tdtdecomposition_gb300.preprocess import group_offsets, preprocess_edges

pytestmark = pytest.mark.gpu


def _small_batch(num=60, seed=3):
    rng = np.random.default_rng(seed)
    graphs = []
    for i in range(num):
        if i % 3 == 0:
            s, d = G.rmat_edges(int(rng.integers(5, 10)), 8 << int(rng.integers(5, 10)), seed=i)
        else:
            s, d = G.ba_edges(int(rng.integers(8, 400)), int(rng.integers(2, 8)), seed=100 + i)
        rows, cols, rp, verts = O.preprocess(np.stack([s, d], 1))
        graphs.append((rows, cols, rp.astype(np.int64)))
    return graphs


def test_batch_equals_each_graph_alone():
    graphs = _small_batch()
    bt = B.pack_host(graphs)
    res = B.decompose(bt)
    for g, (rows, cols, rp) in enumerate(graphs):
        alone = T.truss_decompose(CSRCOO(columns=torch.as_tensor(cols).cuda(), row_ptr=torch.as_tensor(rp).cuda(),
                                         rows=torch.as_tensor(rows).cuda()))
        assert torch.equal(B.per_graph(bt, res, g), alone.truss), g
        assert int(res.kmax[g]) == alone.kmax, g
        if g % 7 == 0:
            V = len(rp) - 1
            kmax, et, pt, tr = O.k_truss(rows, cols, O.tiling_row_ptr(rows, cols, V, 2), V, 2)
            assert np.array_equal(B.per_graph(bt, res, g).cpu().numpy(), tr)


def test_batch_with_device_preprocessing_groups():
    src, dst, vg = W.ba_batch_edges(40, seed=2000)
    g, verts = preprocess_edges(torch.as_tensor(src).cuda(), torch.as_tensor(dst).cuda(), torch.as_tensor(vg).cuda())
    vo, eo = group_offsets(torch.as_tensor(vg).cuda(), verts, g)
    bt = B.batch_from_union(g, eo, vo)
    res = B.decompose(bt)
    n, m = W.ba_batch_params(40, seed=2000)
    off = np.concatenate([[0], np.cumsum(n)])
    vh = verts.cpu().numpy().astype(np.int64)
    rows_h, cols_h = g.rows.cpu().numpy(), g.columns.cpu().numpy()
    tr_h = res.truss.cpu().numpy()
    for i in (0, 7, 39):
        s, d = G.ba_edges(int(n[i]), int(m[i]), 2000 + i)
        r1, c1, rp1, v1 = O.preprocess(np.stack([s, d], 1))
        V1 = len(v1)
        _, _, _, t1 = O.k_truss(r1, c1, O.tiling_row_ptr(r1, c1, V1, 2), V1, 2)
        ref = O.undirected_truss_map(r1, c1, t1, v1)
        a, b = int(eo[i]), int(eo[i + 1])
        got = O.undirected_truss_map(rows_h[a:b], cols_h[a:b], tr_h[a:b], vh - off[i])
        assert got == ref, i


def test_autotune_picks_a_split_and_keeps_results():
    s, d = G.rmat_edges(13, 16 << 13, seed=9)
    rows, cols, rp, verts = O.preprocess(np.stack([s, d], 1))
    g = CSRCOO(columns=torch.as_tensor(cols).cuda(), row_ptr=torch.as_tensor(rp).long().cuda(),
               rows=torch.as_tensor(rows).cuda())
    ref = T.truss_decompose(g, lists=False)
    try:
        cfg = autotune.tune(g)
        assert (cfg.warp_cap, cfg.heavy_cap) in autotune.CANDIDATES
        assert cfg.peel_grid in autotune.PEEL_GRIDS and cfg.vec in autotune.VEC_WALK
        got = T.truss_decompose(g, lists=cfg.lists)
        assert torch.equal(got.truss, ref.truss) and torch.equal(got.e_truss, ref.e_truss)
        # every peel grid and walk width gives the same result
        for pg in autotune.PEEL_GRIDS:
            for vec in autotune.VEC_WALK:
                autotune.apply(autotune.Config(cfg.warp_cap, cfg.heavy_cap, cfg.lists, pg, vec))
                got = T.truss_decompose(g, lists=cfg.lists)
                assert torch.equal(got.truss, ref.truss) and torch.equal(got.e_truss, ref.e_truss), (pg, vec)
        # a cached workload answers without timing
        assert autotune.tune(g) == cfg
    finally:
        autotune.reset()


@pytest.mark.parametrize("list_budget", [None, 0])
def test_captured_batch_replays_equal_the_eager_run(list_budget):
    """A batch recorded once as a CUDA graph (support, listing, the persistent
    cooperative peel and the outputs) and replayed: every replay gives the
    eager run's truss numbers, per-graph kmax and e_truss order; new graphs of
    the same shape copied into the inputs are decomposed by the next replay.
    list_budget 0 captures the search peel (no list tail)."""
    graphs = _small_batch(num=40, seed=11)
    bt = B.pack_host(graphs)
    eager = B.decompose(bt)
    cap = B.capture(bt, list_budget=list_budget)
    for _ in range(2):
        r = cap.replay()
        assert torch.equal(r.truss, eager.truss)
        assert torch.equal(r.kmax, eager.kmax)
        assert torch.equal(r.union.e_truss, eager.union.e_truss)
        assert torch.equal(r.union.ptr_truss, eager.union.ptr_truss)
    # replays re-read the inputs: an invalid CSR copied in is reported by the
    # next replay, and the restored one decomposes again
    saved = bt.graph.columns.clone()
    bt.graph.columns.copy_(bt.graph.rows)
    with pytest.raises(T._lib.TdtError):
        cap.replay()
    bt.graph.columns.copy_(saved)
    assert torch.equal(cap.replay().truss, eager.truss)
