"""The reference's research-variant operators (segment_isinis_m,
segment_isinmm, sub_suppport_affect, peeling_undirect*, peeling_direct_*) and
the undirected-graph drivers built on them (truss_undirect_cuda.py,
truss_undirect_cuda2.py).

CPU: the oracle's restatement of the drivers reproduces the reference's own
recorded peel levels (golden fixtures), and flow.py's drivers follow the same
steps when their operators are the oracle's.  GPU: every operator is bit-exact
against the oracle, and flow.py's drivers on the CUDA operators reproduce the
oracle drivers' e_truss / ptr_truss exactly."""
import types

import numpy as np
import pytest
import torch

from oracle import oracle as O
from oracle import research as R
from tests import _golden as GD
from tdtdecomposition_gb300 import CSRCOO, flow, generators as G

CASES = GD.names()


def _ref_graph(name):
    d = GD.load(name)
    return d, d["ref_rows"].astype(np.int32), d["ref_cols"].astype(np.int32), d["ref_rp"].astype(np.int32), \
        len(d["ref_vertices"])


def _levels(e, p):
    return [set(e[p[i]:p[i + 1]].tolist()) for i in range(len(p) - 1)]


def _oracle_direct(rows, cols, rp, nv, n_cut, thr=10000000):
    rp_t, r_e, re_p = R.preprocess_direct(rows, cols, rp, nv, n_cut)
    return R.undirected_truss_direct(rows, cols, rp_t, r_e, re_p, n_cut, thr)


def _oracle_undirect(rows, cols, rp, nv, n_cut_s, n_cut, thr=10000000):
    dp, cg, nbr, pg = R.preprocess_undirect(rows, cols, rp, nv, n_cut_s, n_cut)
    return R.undirected_truss_undirect(rows, cols, dp, cg, nbr, pg, n_cut_s, n_cut, thr)


# ------------------------------------------------------------------ oracle pin (CPU)
@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("n_cut", [1, 2])
def test_oracle_undirected_drivers_reproduce_reference_levels(name, n_cut):
    """Both drivers peel the same levels the reference's `--cuda` flow
    recorded for the same graph (sg_*1 fixtures: levels from 1, edges without
    triangles in none)."""
    d, rows, cols, rp, nv = _ref_graph(name)
    want_k, want_e, want_p = int(d["sg_kmax1"]), d["sg_e_truss1"], d["sg_ptr_truss1"]
    for thr in (10000000, 64):
        k1, e1, p1 = _oracle_direct(rows, cols, rp, nv, n_cut, thr)
        k2, e2, p2 = _oracle_undirect(rows, cols, rp, nv, n_cut, n_cut, thr)
        assert k1 == k2 == want_k
        assert np.array_equal(p1, want_p) and np.array_equal(p2, want_p)
        assert _levels(e1, p1) == _levels(want_e, want_p)
        assert np.array_equal(e1, e2)


def test_oracle_undirected_drivers_on_rmat_match_k_truss():
    s, t = G.rmat_edges(11, 16 << 11, seed=3)
    rows, cols, rp, verts = O.preprocess(np.stack([s, t], 1))
    nv = len(verts)
    kmax, _, _, truss = O.k_truss(rows, cols, O.tiling_row_ptr(rows, cols, nv, 1), nv, 1)
    k, e, p = _oracle_direct(rows, cols, rp, nv, 3, thr=500)
    assert k == kmax
    assert np.array_equal(GD.truss_from_levels(e, p, len(cols)), truss)


def test_oracle_triangle_free_graph_ends():
    """A graph without triangles: the reference's level search never ends;
    the restatement returns kmax 2 and no levels."""
    rows = np.array([0, 1, 2], np.int32)
    cols = np.array([1, 2, 3], np.int32)
    rp = np.array([0, 1, 2, 3, 3], np.int32)
    k, e, p = _oracle_direct(rows, cols, rp, 4, 1)
    assert k == 2 and len(e) == 0 and list(p) == [0]


def test_oracle_merge_walk_semantics():
    """-1 holes anywhere in a row never match (segment_isinis_m) but do in
    segment_isinmm; matches flag both sides."""
    a = np.array([1, -1, 5, 9, -1, 4, 6], np.int32)
    ap = np.array([0, 4, 7], np.int32)
    b = np.array([-1, 5, 9, 2, 4, 6, 8], np.int32)
    bp = np.array([0, 3, 7], np.int32)
    m1 = np.zeros(7, np.uint8)
    m2 = np.zeros(7, np.uint8)
    R.segment_isinis_m(a, ap, b, bp, m1, m2)
    assert m1.tolist() == [0, 0, 1, 1, 0, 1, 1] and m2.tolist() == [0, 1, 1, 0, 1, 1, 0]
    u = np.array([-1, 3, 7], np.int32)
    v = np.array([-1, 7], np.int32)
    um = np.zeros(3, np.uint8)
    vm = np.zeros(2, np.uint8)
    R.segment_isinmm(u, v, np.array([0, 3], np.int32), np.array([0, 2], np.int32), um, vm)
    assert um.tolist() == [1, 0, 1] and vm.tolist() == [1, 1]


# ------------------------------------------------------------------ flow drivers' host logic (CPU)
def _np(t):
    return t.numpy() if t.dtype != torch.bool else t.numpy().view(np.uint8)


def _oracle_ops():
    """The trusstensor names flow.py's undirected drivers call, served by the
    oracle on CPU tensors (in place through numpy views)."""
    def support(rows, cols, rp, n_cut, out):
        O.segment_isin2tile(_np(rows), _np(cols), _np(rp), n_cut, _np(out))

    def peel(variant, tile):
        def op(e_curr, rows, columns, *rest):
            if tile:
                rest, n_cut = rest[:-1], rest[-1]
            else:
                n_cut = 1
            support, e_mask, n_mark, in_curr, l = rest[-5:]
            lists = rest[:-5]
            kw = {}
            if variant == R.OO:
                kw["row_ptr"] = _np(lists[0])
            elif variant == R.II:
                kw["r_edges"], kw["re_ptr"] = _np(lists[0]), _np(lists[1])
            elif variant == R.OI:
                kw["row_ptr"], kw["r_edges"], kw["re_ptr"] = _np(lists[0]), _np(lists[1]), _np(lists[2])
            else:
                kw["columns_g"], kw["row_ptr"], kw["edges_id_nbr"] = _np(lists[0]), _np(lists[1]), _np(lists[2])
            R.peel_op(variant, _np(e_curr), _np(rows), _np(columns), _np(support), _np(e_mask), _np(n_mark),
                      _np(in_curr), l, n_cut, **kw)
        return op

    return types.SimpleNamespace(
        segment_add=lambda c, p, o: O.segment_add(_np(c), _np(p), _np(o)),
        segment_isin2=lambda r, c, p, o: support(r, c, p, 1, o),
        segment_isin2tile=lambda r, c, p, n, o: support(r, c, p, n, o),
        peeling_direct_oo=peel(R.OO, False), peeling_direct_tile_oo=peel(R.OO, True),
        peeling_direct_ii=peel(R.II, False), peeling_direct_tile_ii=peel(R.II, True),
        peeling_direct_oi=peel(R.OI, False), peeling_direct_tile_oi=peel(R.OI, True),
        peeling_undirect=peel(R.UNDIRECT, False), peeling_undirect_tile=peel(R.UNDIRECT, True))


@pytest.mark.parametrize("n_cut", [1, 3])
def test_flow_undirected_drivers_follow_the_oracle_steps(monkeypatch, n_cut):
    monkeypatch.setattr(flow, "tt", _oracle_ops())
    s, t = G.rmat_edges(10, 16 << 10, seed=5)
    rows, cols, rp, verts = O.preprocess(np.stack([s, t], 1))
    nv = len(verts)
    g = CSRCOO(columns=torch.as_tensor(cols, dtype=torch.int32), row_ptr=torch.as_tensor(rp, dtype=torch.int64),
               rows=torch.as_tensor(rows, dtype=torch.int32))
    for thr in (10000000, 300):
        want = _oracle_direct(rows, cols, rp, nv, n_cut, thr)
        rp_t, r_e, re_p = flow.preprocess_direct(g, n_cut)
        o_rp, o_r, o_re = R.preprocess_direct(rows, cols, rp, nv, n_cut)
        assert np.array_equal(rp_t.numpy(), o_rp) and np.array_equal(r_e.numpy(), o_r)
        assert np.array_equal(re_p.numpy(), o_re)
        got = flow.undirected_truss_direct(g, rp_t, r_e, re_p, n_cut, thr)
        assert got[0] == want[0]
        assert np.array_equal(got[1].numpy(), want[1]) and np.array_equal(got[2].numpy(), want[2])
        parts = flow.preprocess_undirect(g, 2, n_cut)
        o_parts = R.preprocess_undirect(rows, cols, rp, nv, 2, n_cut)
        for a, b in zip(parts, o_parts):
            assert np.array_equal(a.numpy(), b)
        got = flow.undirected_truss_undirect(g, parts[1], parts[2], parts[0], parts[3], 2, n_cut, thr)
        assert got[0] == want[0]
        assert np.array_equal(got[1].numpy(), want[1]) and np.array_equal(got[2].numpy(), want[2])
    # the caller's graph is left as it was
    assert np.array_equal(g.columns.numpy(), cols)


# ------------------------------------------------------------------ CUDA operators (GPU)
def _cu(a, dtype=torch.int32):
    return torch.as_tensor(np.ascontiguousarray(a)).to(dtype).cuda()


def _host(t):
    return t.cpu().numpy().astype(np.uint8) if t.dtype == torch.bool else t.cpu().numpy()


def _sorted_rows(rng, n_rows, max_len, universe, holes):
    lens = rng.integers(0, max_len + 1, n_rows)
    vals = [np.sort(rng.choice(universe, size=k, replace=False)) for k in lens]
    cols = np.concatenate(vals).astype(np.int32) if n_rows else np.zeros(0, np.int32)
    if holes:
        cols[rng.random(cols.shape[0]) < holes] = -1
    ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    return cols, ptr


def _messy(rng, cols, ptr, shape):
    """Rows the reference's merge still walks, but not strictly increasing."""
    cols = cols.copy()
    if shape == "holes":
        cols[rng.random(cols.shape[0]) < 0.1] = -1
    elif shape == "shuffled":
        for r in range(len(ptr) - 1):
            if rng.random() < 0.3:
                rng.shuffle(cols[ptr[r]:ptr[r + 1]])
    elif shape == "dups":
        d = rng.random(cols.shape[0]) < 0.2
        d[ptr[:-1][ptr[:-1] < cols.shape[0]]] = False
        cols[d] = np.roll(cols, 1)[d]
    return cols


@pytest.mark.gpu
@pytest.mark.parametrize("shape", ["sorted", "holes", "shuffled", "dups"])
@pytest.mark.parametrize("max_len", [6, 90, 700])
def test_segment_isinis_m_and_isinmm_gpu(max_len, shape):
    """Both row-wise match ops give the reference's merge-walk marks: sorted
    rows (hash path) and rows with -1 holes, shuffled rows and repeated values
    (one-lane merge, or the hash path where the holes are isinis_m's)."""
    from tdtdecomposition_gb300 import trusstensor as tt
    rng = np.random.default_rng(max_len)
    n = 3000 if max_len < 100 else 300
    # segment_isinis_m takes (a, a_ptr, b, b_ptr), segment_isinmm (u, v, u_ptr, v_ptr)
    for ora, op, order in ((R.segment_isinis_m, tt.segment_isinis_m, (0, 1, 2, 3)),
                           (R.segment_isinmm, tt.segment_isinmm, (0, 2, 1, 3))):
        a, ap = _sorted_rows(rng, n, max_len, 2 * max_len + 5, 0.0)
        b, bp = _sorted_rows(rng, n, max_len, 2 * max_len + 5, 0.0)
        a, b = _messy(rng, a - 3, ap, shape), _messy(rng, b - 3, bp, shape)
        args = [(a, ap, b, bp)[i] for i in order]
        m1, m2 = np.zeros(len(a), np.uint8), np.zeros(len(b), np.uint8)
        ora(*args, m1, m2)
        g1 = torch.zeros(len(a), dtype=torch.bool, device="cuda")
        g2 = torch.zeros(len(b), dtype=torch.bool, device="cuda")
        op(*[_cu(x) for x in args], g1, g2)
        assert m1.any()
        assert np.array_equal(_host(g1), m1) and np.array_equal(_host(g2), m2)


@pytest.mark.gpu
def test_sub_suppport_affect_gpu():
    from tdtdecomposition_gb300 import trusstensor as tt
    rng = np.random.default_rng(7)
    E, n = 5000, 200000
    left = rng.integers(0, E, n).astype(np.int32)
    right = rng.integers(0, E, n).astype(np.int32)
    cur = rng.integers(0, E, n).astype(np.int32)
    m1 = (rng.random(n) < 0.6).astype(np.uint8)
    m2 = (rng.random(n) < 0.6).astype(np.uint8)
    sup = rng.integers(0, 400, E).astype(np.int32)
    want_s, want_a = sup.copy(), np.zeros(E, np.uint8)
    R.sub_suppport_affect(left, right, cur, want_s, m1, m2, want_a, 3)
    gs = _cu(sup)
    ga = torch.zeros(E, dtype=torch.bool, device="cuda")
    tt.sub_suppport_affect(_cu(left), _cu(right), _cu(cur), gs, _cu(m1, torch.bool), _cu(m2, torch.bool), ga, 3)
    assert np.array_equal(_host(gs), want_s) and np.array_equal(_host(ga), want_a)


def _peel_case(seed, scale, n_cut):
    s, t = G.rmat_edges(scale, 16 << scale, seed=seed)
    rows, cols, rp, verts = O.preprocess(np.stack([s, t], 1))
    nv = len(verts)
    rng = np.random.default_rng(seed)
    sup = O.support(rows, cols, O.tiling_row_ptr(rows, cols, nv, 1), 1).astype(np.int32)
    E = len(cols)
    e_mask = (rng.random(E) < 0.9).astype(np.uint8)
    in_curr = (rng.random(E) < 0.05).astype(np.uint8) & e_mask
    e_curr = np.nonzero(in_curr)[0].astype(np.int32)
    l = int(np.median(sup[sup > 0])) if (sup > 0).any() else 1
    return rows, cols, rp, nv, sup, e_mask, in_curr, e_curr, l


@pytest.mark.gpu
@pytest.mark.parametrize("n_cut", [1, 3])
@pytest.mark.parametrize("variant", ["oo", "ii", "oi", "undirect"])
def test_peel_operators_gpu(variant, n_cut):
    from tdtdecomposition_gb300 import trusstensor as tt
    rows, cols, rp, nv, sup, e_mask, in_curr, e_curr, l = _peel_case(11, 12, n_cut)
    E = len(cols)
    want_s, want_m = sup.copy(), np.zeros(E, np.uint8)
    gs, gm = _cu(sup), torch.zeros(E, dtype=torch.bool, device="cuda")
    common = (_cu(e_curr), _cu(rows), _cu(cols))
    tail = (gs, _cu(e_mask, torch.bool), gm, _cu(in_curr, torch.bool), l)
    if variant == "undirect":
        dp, cg, nbr, pg = R.preprocess_undirect(rows, cols, rp, nv, 1, n_cut)
        R.peel_op(R.UNDIRECT, e_curr, rows, cols, want_s, e_mask, want_m, in_curr, l, n_cut, row_ptr=pg,
                  columns_g=cg, edges_id_nbr=nbr)
        lists = (_cu(cg), _cu(pg), _cu(nbr))
        fn = tt.peeling_undirect_tile if n_cut > 1 else tt.peeling_undirect
    else:
        rp_t, r_e, re_p = R.preprocess_direct(rows, cols, rp, nv, n_cut)
        v = {"oo": R.OO, "ii": R.II, "oi": R.OI}[variant]
        R.peel_op(v, e_curr, rows, cols, want_s, e_mask, want_m, in_curr, l, n_cut, row_ptr=rp_t, r_edges=r_e,
                  re_ptr=re_p)
        lists = {"oo": (_cu(rp_t),), "ii": (_cu(r_e), _cu(re_p)), "oi": (_cu(rp_t), _cu(r_e), _cu(re_p))}[variant]
        fn = getattr(tt, "peeling_direct_%s%s" % ("tile_" if n_cut > 1 else "", variant))
    fn(*common, *lists, *tail, *((n_cut,) if n_cut > 1 else ()))
    assert (want_s != sup).any()
    assert np.array_equal(_host(gs), want_s)
    assert np.array_equal(_host(gm), want_m)


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["oo", "ii", "undirect"])
def test_peel_operators_on_unsorted_lists_gpu(variant):
    """Lists out of order (shuffled in-lists, shuffled symmetric adjacency,
    shuffled out-lists): the one-lane merge path gives the reference's
    decrements and marks."""
    from tdtdecomposition_gb300 import trusstensor as tt
    rows, cols, rp, nv, sup, e_mask, in_curr, e_curr, l = _peel_case(5, 11, 1)
    rng = np.random.default_rng(1)
    E = len(cols)
    want_s, want_m = sup.copy(), np.zeros(E, np.uint8)
    gs, gm = _cu(sup), torch.zeros(E, dtype=torch.bool, device="cuda")
    if variant == "undirect":
        dp, cg, nbr, pg = R.preprocess_undirect(rows, cols, rp, nv, 1, 1)
        perm = np.arange(len(cg))
        for v in range(nv):
            if rng.random() < 0.3:
                rng.shuffle(perm[pg[v]:pg[v + 1]])
        cg, nbr = cg[perm], nbr[perm]
        R.peel_op(R.UNDIRECT, e_curr, rows, cols, want_s, e_mask, want_m, in_curr, l, 1, row_ptr=pg, columns_g=cg,
                  edges_id_nbr=nbr)
        tt.peeling_undirect(_cu(e_curr), _cu(rows), _cu(cols), _cu(cg), _cu(pg), _cu(nbr), gs,
                            _cu(e_mask, torch.bool), gm, _cu(in_curr, torch.bool), l)
    else:
        rp_t, r_e, re_p = R.preprocess_direct(rows, cols, rp, nv, 1)
        if variant == "ii":
            for v in range(nv):
                if rng.random() < 0.3:
                    rng.shuffle(r_e[re_p[v]:re_p[v + 1]])
            R.peel_op(R.II, e_curr, rows, cols, want_s, e_mask, want_m, in_curr, l, 1, r_edges=r_e, re_ptr=re_p)
            tt.peeling_direct_ii(_cu(e_curr), _cu(rows), _cu(cols), _cu(r_e), _cu(re_p), gs,
                                 _cu(e_mask, torch.bool), gm, _cu(in_curr, torch.bool), l)
        else:
            cols = cols.copy()
            for v in range(nv):
                if rng.random() < 0.3:
                    rng.shuffle(cols[rp_t[v]:rp_t[v + 1]])
            R.peel_op(R.OO, e_curr, rows, cols, want_s, e_mask, want_m, in_curr, l, 1, row_ptr=rp_t)
            tt.peeling_direct_oo(_cu(e_curr), _cu(rows), _cu(cols), _cu(rp_t), gs, _cu(e_mask, torch.bool), gm,
                                 _cu(in_curr, torch.bool), l)
    assert (want_s != sup).any()
    assert np.array_equal(_host(gs), want_s)
    assert np.array_equal(_host(gm), want_m)


@pytest.mark.gpu
def test_peel_operators_reject_bad_calls_gpu():
    from tdtdecomposition_gb300 import trusstensor as tt
    rows, cols, rp, nv, sup, e_mask, in_curr, e_curr, l = _peel_case(3, 8, 1)
    rp_t = _cu(rp)
    with pytest.raises(ValueError):   # support shorter than the edge list
        tt.peeling_direct_oo(_cu(e_curr), _cu(rows), _cu(cols), rp_t, _cu(sup[:-1]), _cu(e_mask, torch.bool),
                             torch.zeros(len(cols), dtype=torch.bool, device="cuda"), _cu(in_curr, torch.bool), l)
    with pytest.raises(TypeError):    # int64 e_curr
        tt.peeling_direct_oo(_cu(e_curr, torch.int64), _cu(rows), _cu(cols), rp_t, _cu(sup),
                             _cu(e_mask, torch.bool), torch.zeros(len(cols), dtype=torch.bool, device="cuda"),
                             _cu(in_curr, torch.bool), l)
    # an empty current set is a no-op
    gs = _cu(sup)
    tt.peeling_direct_oo(_cu(np.zeros(0, np.int32)), _cu(rows), _cu(cols), rp_t, gs, _cu(e_mask, torch.bool),
                         torch.zeros(len(cols), dtype=torch.bool, device="cuda"), _cu(in_curr, torch.bool), l)
    assert np.array_equal(_host(gs), sup)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("n_cut", [1, 2])
def test_flow_undirected_drivers_gpu(name, n_cut):
    d, rows, cols, rp, nv = _ref_graph(name)
    g = CSRCOO(columns=_cu(cols), row_ptr=_cu(rp, torch.int64), rows=_cu(rows))
    want = _oracle_direct(rows, cols, rp, nv, n_cut, thr=256)
    got = flow.undirected_truss_direct(g, *flow.preprocess_direct(g, n_cut), n_cut, compact_threshold=256)
    assert got[0] == want[0] == int(d["sg_kmax1"])
    assert np.array_equal(_host(got[1]), want[1]) and np.array_equal(_host(got[2]), want[2])
    dp, cg, nbr, pg = flow.preprocess_undirect(g, n_cut, n_cut)
    got = flow.undirected_truss_undirect(g, cg, nbr, dp, pg, n_cut, n_cut, compact_threshold=256)
    assert got[0] == want[0]
    assert np.array_equal(_host(got[1]), want[1]) and np.array_equal(_host(got[2]), want[2])


@pytest.mark.gpu
def test_flow_undirected_direct_matches_decomposition_gpu():
    """A larger R-MAT graph: the oriented-peel driver's truss numbers equal the
    device-resident decomposition's."""
    from tdtdecomposition_gb300 import truss as T
    s, t = G.rmat_edges(16, 16 << 16, seed=9)
    rows, cols, rp, verts = O.preprocess(np.stack([s, t], 1))
    g = CSRCOO(columns=_cu(cols), row_ptr=_cu(rp, torch.int64), rows=_cu(rows))
    k, e, p = flow.undirected_truss_direct(g, *flow.preprocess_direct(g, 2), 2, compact_threshold=100000)
    res = T.truss_decompose(g)
    assert k == res.kmax
    assert np.array_equal(GD.truss_from_levels(_host(e), _host(p), len(cols)), _host(res.truss))


# ------------------------------------------------------------------ fusion ablation ("before" flows)
def _isinmm_ops():
    return types.SimpleNamespace(
        segment_add=lambda c, p, o: O.segment_add(_np(c), _np(p), _np(o)),
        segment_isinmm=lambda u, v, up, vp, um, vm: R.segment_isinmm(_np(u), _np(v), _np(up), _np(vp), _np(um),
                                                                     _np(vm)))


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("n_cut,compact", [(1, 1000000), (2, 1000000), (2, 0)])
def test_unfused_flow_reproduces_reference_peel_order(monkeypatch, name, n_cut, compact):
    """k_truss(fused=False): support_computing_before and
    all_affect_support_not_before (fusionexperiental.py:24-67) over the
    oracle's segment_isinmm / segment_add give the reference's recorded
    e_truss / ptr_truss exactly."""
    monkeypatch.setattr(flow, "tt", _isinmm_ops())
    d = GD.load(name)
    V = d["ref_vertices"].shape[0]
    g = CSRCOO(columns=torch.as_tensor(d["ref_cols"], dtype=torch.int32),
               row_ptr=torch.as_tensor(d["ref_rp_tiled%d" % n_cut], dtype=torch.int32),
               rows=torch.as_tensor(d["ref_rows"], dtype=torch.int32))
    sup = flow.support_computing_before(g.rows, g.columns, g.row_ptr, n_cut)
    assert np.array_equal(sup.numpy(), d["ref_support"])
    kmax, et, pt = flow.k_truss(g, n_cut, V, compact_threshold=compact, fused=False)
    assert kmax == int(d["sg_kmax%d" % n_cut])
    assert np.array_equal(et.numpy(), d["sg_e_truss%d" % n_cut])
    assert np.array_equal(pt.numpy(), d["sg_ptr_truss%d" % n_cut])


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_unfused_flow_gpu(name):
    d = GD.load(name)
    V = d["ref_vertices"].shape[0]
    g = CSRCOO(columns=_cu(d["ref_cols"]), row_ptr=_cu(d["ref_rp_tiled2"]), rows=_cu(d["ref_rows"]))
    sup = flow.support_computing_before(g.rows, g.columns, g.row_ptr, 2)
    assert np.array_equal(_host(sup), d["ref_support"])
    kmax, et, pt = flow.k_truss(g, 2, V, fused=False)
    assert kmax == int(d["sg_kmax2"])
    assert np.array_equal(_host(et), d["sg_e_truss2"])
    assert np.array_equal(pt.numpy(), d["sg_ptr_truss2"])


@pytest.mark.gpu
def test_unfused_support_matches_fused_on_rmat_gpu():
    s, t = G.rmat_edges(15, 16 << 15, seed=4)
    rows, cols, rp, verts = O.preprocess(np.stack([s, t], 1))
    rp32 = _cu(rp)
    a = flow.support_computing(_cu(rows), _cu(cols), rp32, 1)
    b = flow.support_computing_before(_cu(rows), _cu(cols), rp32, 1)
    assert torch.equal(a, b) and int(a.sum()) > 0


# ------------------------------------------------------------------ tensor_original driver
@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("thr", [100000, 40])
def test_oracle_tensor_original_reproduces_reference_levels(name, thr):
    """truss_nosavetri_tensor4.py's driver (segment_isinis_m + sub_suppport_affect)
    peels the reference's recorded sub-rounds in order; as written there, the
    edges of its last sub-round never reach e_truss."""
    d, rows, cols, rp, nv = _ref_graph(name)
    srp, sc = R.symmetric_csr(rows, cols, nv)
    e, p = R.truss_tensor_original(srp, sc, thr)
    want_e, want_p = d["sg_e_truss1"], d["sg_ptr_truss1"]
    assert len(p) == len(want_p) and np.array_equal(p[:-1], want_p[:-1])
    assert p[-1] == len(e) and np.array_equal(e, want_e[:len(e)])


def _tensor_original_ops():
    def support(rows, cols, rp, out):
        O.segment_isin2tile(_np(rows), _np(cols), _np(rp), 1, _np(out))

    return types.SimpleNamespace(
        segment_add=lambda c, p, o: O.segment_add(_np(c), _np(p), _np(o)),
        segment_isin2=support,
        segment_isinis_m=lambda a, ap, b, bp, m1, m2: R.segment_isinis_m(_np(a), _np(ap), _np(b), _np(bp), _np(m1),
                                                                         _np(m2)),
        sub_suppport_affect=lambda ln, rn, cr, s, m1, m2, af, l: R.sub_suppport_affect(
            _np(ln), _np(rn), _np(cr), _np(s), _np(m1), _np(m2), _np(af), l))


@pytest.mark.parametrize("thr", [100000, 300])
def test_flow_tensor_original_follows_the_oracle_steps(monkeypatch, thr):
    monkeypatch.setattr(flow, "tt", _tensor_original_ops())
    s, t = G.rmat_edges(10, 16 << 10, seed=6)
    rows, cols, rp, verts = O.preprocess(np.stack([s, t], 1))
    nv = len(verts)
    g = CSRCOO(columns=torch.as_tensor(cols, dtype=torch.int32), row_ptr=torch.as_tensor(rp, dtype=torch.int64),
               rows=torch.as_tensor(rows, dtype=torch.int32))
    srp, sc = flow.symmetric_csr(g)
    o_rp, o_c = R.symmetric_csr(rows, cols, nv)
    assert np.array_equal(srp.numpy(), o_rp) and np.array_equal(sc.numpy(), o_c)
    e, p = flow.truss_tensor_original(srp, sc, thr)
    we, wp = R.truss_tensor_original(o_rp, o_c, thr)
    assert np.array_equal(e.numpy(), we) and np.array_equal(p.numpy(), wp)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_flow_tensor_original_gpu(name):
    d, rows, cols, rp, nv = _ref_graph(name)
    g = CSRCOO(columns=_cu(cols), row_ptr=_cu(rp, torch.int64), rows=_cu(rows))
    srp, sc = flow.symmetric_csr(g)
    e, p = flow.truss_tensor_original(srp, sc, compact_threshold=200)
    we, wp = R.truss_tensor_original(*R.symmetric_csr(rows, cols, nv), 200)
    assert np.array_equal(_host(e), we) and np.array_equal(p.numpy(), wp)
