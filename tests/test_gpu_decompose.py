"""Device-resident decomposition, k-truss search and triangle count through
the C ABI, against the reference's golden outputs and the oracle."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests import _golden as GD
from tdtdecomposition_gb300 import CSRCOO, _lib, generators as G, truss as T
from tdtdecomposition_gb300._lib import TdtError

pytestmark = pytest.mark.gpu
CASES = GD.names()


def graph_of(rows, cols, rp):
    return CSRCOO(columns=torch.as_tensor(cols, dtype=torch.int32).cuda(),
                  row_ptr=torch.as_tensor(np.asarray(rp), dtype=torch.int64).cuda(),
                  rows=torch.as_tensor(rows, dtype=torch.int32).cuda())


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("lists", [True, False])
def test_decompose_matches_reference_peel_order(name, lists):
    """Both peel modes: triangles read from per-edge lists, or found by search."""
    d = GD.load(name)
    g = graph_of(d["ref_rows"], d["ref_cols"], d["ref_rp"])
    res = T.truss_decompose(g, lists=lists)
    assert res.listed == (lists and int(d["ref_support"].sum()) > 0)
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
@pytest.mark.parametrize("lists", [True, False])
def test_ktruss_search_matches_reference(name, lists):
    d = GD.load(name)
    g = graph_of(d["ref_rows"], d["ref_cols"], d["ref_rp"])
    truss = GD.truss_from_levels(d["sg_e_truss2"], d["sg_ptr_truss2"], d["ref_cols"].shape[0])
    for k in list(d["kt_ks"]) + [1, 2]:
        m = T.ktruss_search(g, int(k), lists=lists).cpu().numpy()
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
    g = graph_of(rows, cols, rp)
    for lists in (True, False):
        res = T.truss_decompose(g, lists=lists)
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


def test_list_capacity_fallback():
    """A workspace tail too small for the lists falls back to the search peel
    on the device, with identical results."""
    from tdtdecomposition_gb300 import _lib
    s, d = G.rmat_edges(12, 16 << 12, seed=3)
    rows, cols, rp, verts = O.preprocess(np.stack([s, d], 1))
    g = graph_of(rows, cols, rp)
    full = T.truss_decompose(g, lists=True)
    L = _lib.load()
    V, E = len(verts), len(cols)
    base = (L.tdt_decompose_workspace_bytes(V, E) + 255) // 256 * 256
    ws = T.Workspace()
    ws.buf = torch.empty(base + 1024, dtype=torch.uint8, device="cuda")  # tail of 1 KB: too small
    ws.triangles[T._graph_key(g.columns, g.row_ptr.long())] = 1
    small = T.truss_decompose(g, workspace=ws, lists=True)
    assert torch.equal(full.truss, small.truss) and torch.equal(full.e_truss, small.e_truss)


def test_repeatable_and_workspace_reuse():
    s, d = G.rmat_edges(13, 16 << 13, seed=21)
    rows, cols, rp, verts = O.preprocess(np.stack([s, d], 1))
    g = graph_of(rows, cols, rp)
    ws = T.Workspace()
    a = T.truss_decompose(g, workspace=ws)
    b = T.truss_decompose(g, workspace=ws)
    assert torch.equal(a.truss, b.truss) and torch.equal(a.e_truss, b.e_truss)


@pytest.mark.parametrize("vec,bulk", [(1, 0), (1, 1), (0, 0)])
@pytest.mark.parametrize("caps", [(4, 16), (8, 10 ** 6), (2, 3)])
def test_all_support_paths_vs_oracle(caps, vec, bulk):
    """Lowered light/heavy thresholds push small graphs through the block-level
    heavy-row walk and the in-place (beyond shared memory) path, with the
    wedge walk over 16-byte column chunks and over single columns, and the
    heavy rows staged by plain loads or by a bulk copy."""
    from tdtdecomposition_gb300 import _lib
    L = _lib.load()
    s, d = G.rmat_edges(12, 16 << 12, seed=31)
    pairs = np.stack([s, d], 1)
    rows, cols, rp, verts = O.preprocess(pairs)
    sup_ref = O.support(rows, cols, rp.astype(np.int32), 1)
    L.tdt_set_support_caps(*caps)
    L.tdt_set_vector_walk(vec)
    L.tdt_set_bulk_staging(bulk)
    try:
        t, sup = T.triangle_count(graph_of(rows, cols, rp), return_support=True)
        assert np.array_equal(sup.cpu().numpy(), sup_ref)
        _oracle_check(pairs)
        # the drop-in operator (accumulate mode, int32 offsets, any orientation)
        from tdtdecomposition_gb300 import trusstensor as tt
        out = torch.zeros(len(cols), dtype=torch.int32, device="cuda")
        tt.segment_isin2(torch.as_tensor(rows).cuda(), torch.as_tensor(cols).cuda(),
                         torch.as_tensor(rp.astype(np.int32)).cuda(), out)
        assert np.array_equal(out.cpu().numpy(), sup_ref)
    finally:
        L.tdt_set_support_caps(0, 0)
        L.tdt_set_vector_walk(1)
        L.tdt_set_bulk_staging(0)


def test_unaligned_columns_take_the_scalar_walk():
    """The drop-in operator on a columns array that starts 4 bytes past a
    16-byte boundary (the vectorised walk needs 16-byte alignment) gives the
    oracle's support."""
    from tdtdecomposition_gb300 import trusstensor as tt
    s, d = G.rmat_edges(11, 16 << 11, seed=8)
    rows, cols, rp, verts = O.preprocess(np.stack([s, d], 1))
    sup_ref = O.support(rows, cols, rp.astype(np.int32), 1)
    buf = torch.zeros(len(cols) + 1, dtype=torch.int32, device="cuda")
    buf[1:] = torch.as_tensor(cols).cuda()
    c1 = buf[1:]
    assert c1.data_ptr() % 16 != 0
    out = torch.zeros(len(cols), dtype=torch.int32, device="cuda")
    tt.segment_isin2(torch.as_tensor(rows).cuda(), c1, torch.as_tensor(rp.astype(np.int32)).cuda(), out)
    assert np.array_equal(out.cpu().numpy(), sup_ref)


@pytest.mark.parametrize("route", [2, 1, 0])
def test_listing_routes_vs_oracle(route):
    """The three ways the peel gets each edge's triangles, chosen by the list
    tail: one walk that counts and lists (tail = lists + staging), a count
    walk then a listing walk (tail = lists only), and the search peel (no
    tail).  All three give the oracle's e_truss / ptr_truss."""
    s, d = G.rmat_edges(13, 16 << 13, seed=12)
    pairs = np.stack([s, d], 1)
    rows, cols, rp, verts = O.preprocess(pairs)
    V = len(verts)
    kmax, et, pt, truss = O.k_truss(rows, cols, O.tiling_row_ptr(rows, cols, V, 1), V, 1)
    g = graph_of(rows, cols, rp)
    tri = T.triangle_count(g)
    stage = T.stage_bytes(g.columns, g.row_ptr, g.rows)
    budget = {2: 24 * tri + stage + 256, 1: 24 * tri + 256, 0: 0}[route]
    res = T.truss_decompose(g, list_budget=budget)
    assert res.listing == route
    assert res.kmax == kmax
    assert np.array_equal(res.truss.cpu().numpy(), truss)
    assert np.array_equal(res.e_truss.cpu().numpy(), et)
    assert np.array_equal(res.ptr_truss.cpu().numpy(), pt)
    ks = T.ktruss_search(g, max(3, kmax // 2), lists=True)
    assert np.array_equal(ks.cpu().numpy(), truss >= max(3, kmax // 2))


def test_deterministic_at_scale():
    """R-MAT scale 17 (rows above the warp threshold): two runs agree, and
    agree with the oracle."""
    s, d = G.rmat_edges(17, 16 << 17, seed=1)
    pairs = np.stack([s, d], 1)
    rows, cols, rp, verts = O.preprocess(pairs)
    assert np.diff(rp).max() > 256
    g = graph_of(rows, cols, rp)
    a = T.truss_decompose(g, lists=True)
    b = T.truss_decompose(g, lists=True)
    c = T.truss_decompose(g, lists=False)
    assert torch.equal(a.truss, b.truss) and torch.equal(a.e_truss, b.e_truss)
    assert torch.equal(a.truss, c.truss) and torch.equal(a.e_truss, c.e_truss)
    _oracle_check(pairs)


def _books(copies, k, pages, seed=0):
    """copies of K_k with `pages` extra vertices glued to every clique edge:
    each glued edge lies in one triangle, so level 1 queues long runs of
    edges owning a single triangle-list slot each."""
    rng = np.random.default_rng(seed)
    edges, base = [], 0
    for _ in range(copies):
        nxt = base + k
        for a in range(k):
            for b in range(a + 1, k):
                edges.append((base + a, base + b))
                for _ in range(pages):
                    edges += [(base + a, nxt), (base + b, nxt)]
                    nxt += 1
        base = nxt
    perm = rng.permutation(base)
    return perm[np.array(edges, dtype=np.int64)].astype(np.int32)


def test_listed_peel_long_runs_of_unit_items():
    """336K frontier edges with one list slot each: every warp walks several
    windows of single-slot items (regression test of the window advance)."""
    pairs = _books(2000, 8, 3)
    _oracle_check(pairs)
    rows, cols, rp, verts = O.preprocess(pairs)
    g = graph_of(rows, cols, rp)
    a = T.truss_decompose(g, lists=True)
    b = T.truss_decompose(g, lists=True)
    assert torch.equal(a.truss, b.truss) and torch.equal(a.e_truss, b.e_truss)


def test_level_gaps_vs_oracle():
    """Disjoint cliques K_4, K_9, K_40, K_120, K_230 plus a sparse random
    part: consecutive levels, gaps inside the level-change side window
    (64) and gaps beyond it."""
    rng = np.random.default_rng(11)
    edges, base = [], 0
    for k in (4, 9, 40, 120, 230):
        a, b = np.triu_indices(k, 1)
        edges.append(np.stack([a + base, b + base], 1))
        base += k
    n = 3000
    edges.append(rng.integers(base, base + n, size=(12000, 2)))
    pairs = np.concatenate(edges).astype(np.int32)
    pairs = rng.permutation(base + n).astype(np.int32)[pairs]
    _oracle_check(pairs)


@pytest.mark.parametrize("caps", [(64, 1 << 30), (1 << 20, 300), (1, 1)])
@pytest.mark.parametrize("lists", [True, False])
def test_ktruss_search_in_small_batches(caps, lists):
    """k-truss search whose starting frontier is queued a few edges (or a few
    candidate slots) per sub-round: the same edge sets as without batching."""
    from tdtdecomposition_gb300 import _lib
    L = _lib.load()
    s, d = G.rmat_edges(11, 16 << 11, seed=21)
    rows, cols, rp, verts = O.preprocess(np.stack([s, d], 1))
    g = graph_of(rows, cols, rp)
    truss = T.truss_decompose(g).truss.cpu().numpy()
    L.tdt_set_ktruss_batch_caps(*caps)
    try:
        for k in (3, 4, 6, int(truss.max()), int(truss.max()) + 1):
            m = T.ktruss_search(g, k, lists=lists).cpu().numpy()
            assert np.array_equal(m, truss >= k), (caps, k)
    finally:
        L.tdt_set_ktruss_batch_caps(0, 0)


@pytest.mark.parametrize("scale", [12, 15])
def test_search_peel_dynamic_ranges(scale):
    """The peel without lists, with every sub-round split into dynamic 256-slot
    ranges (the default only splits sub-rounds of 2^20+ slots): the same truss
    numbers and peel order as the listed peel and the static split."""
    s, d = G.rmat_edges(scale, 16 << scale, seed=3)
    rows, cols, rp, verts = O.preprocess(np.stack([s, d], 1))
    g = graph_of(rows, cols, rp)
    L = _lib.load()
    ref = T.truss_decompose(g, lists=True)
    static = T.truss_decompose(g, lists=False)
    L.tdt_set_peel_dynamic_min(64)
    try:
        dyn = T.truss_decompose(g, lists=False)
        kt = T.ktruss_search(g, max(3, ref.kmax // 2), lists=False)
    finally:
        L.tdt_set_peel_dynamic_min(0)
    assert not dyn.listed and ref.listed
    for r in (static, dyn):
        assert r.kmax == ref.kmax and torch.equal(r.truss, ref.truss) and torch.equal(r.e_truss, ref.e_truss)
    assert torch.equal(kt, ref.truss >= max(3, ref.kmax // 2))


def test_phase_profile_and_peel_clock():
    """Phase times (CUDA events on the call's stream) of two decompositions,
    and block 0's clock of the last peel."""
    s, d = G.rmat_edges(12, 16 << 12, seed=1)
    rows, cols, rp, verts = O.preprocess(np.stack([s, d], 1))
    g = graph_of(rows, cols, rp)
    ws = T.Workspace()
    T.truss_decompose(g, workspace=ws)
    with T.PhaseProfile() as prof:
        for _ in range(2):
            res = T.truss_decompose(g, workspace=ws)
    assert res.listed and prof.calls == 2
    assert all(prof.ms[p] > 0 for p in T.PHASES)
    clk = T.peel_clock(ws)
    assert 0 < clk["processing"] <= clk["total"]
    assert clk["barrier_waits"] >= 0 and clk["level_changes"] >= 0
