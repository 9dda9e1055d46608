"""Drop-in trusstensor operators on the GPU against the oracle (bit-exact on
everything the reference computes deterministically)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests import _golden as GD
from tdtdecomposition_gb300 import flow, trusstensor as tt, CSRCOO

pytestmark = pytest.mark.gpu
CASES = GD.names()


def cu(a, dtype=torch.int32):
    return torch.as_tensor(np.ascontiguousarray(a)).to(dtype).cuda()


def host(t):
    return t.cpu().numpy()


def _rand_graph(seed, V=400, m=5000):
    rng = np.random.default_rng(seed)
    pairs = np.stack([rng.integers(0, V, m), rng.integers(0, V, m)], 1).astype(np.int32)
    return O.preprocess(pairs, stable=True)


def test_segment_add():
    rng = np.random.default_rng(0)
    ptr = np.concatenate([[0], np.cumsum(rng.integers(0, 5, 1000))]).astype(np.int32)
    vals = rng.integers(-3, 4, ptr[-1]).astype(np.int32)
    a = np.full(1000, 7, np.int32)
    O.segment_add(vals, ptr, a)
    out = cu(np.full(1000, 7, np.int32))
    tt.segment_add(cu(vals), cu(ptr), out)
    assert np.array_equal(host(out), a)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("n_cut", [1, 2, 3])
def test_segment_isin2tile_matches_reference_support(name, n_cut):
    d = GD.load(name)
    V = d["ref_vertices"].shape[0]
    rpt = O.tiling_row_ptr(d["ref_rows"], d["ref_cols"], V, n_cut)
    out = torch.zeros(d["ref_cols"].shape[0], dtype=torch.int32, device="cuda")
    if n_cut == 1:
        tt.segment_isin2(cu(d["ref_rows"]), cu(d["ref_cols"]), cu(rpt), out)
    else:
        tt.segment_isin2tile(cu(d["ref_rows"]), cu(d["ref_cols"]), cu(rpt), n_cut, out)
    assert np.array_equal(host(out), d["ref_support"])
    # accumulates, like the reference
    tt.segment_isin2tile(cu(d["ref_rows"]), cu(d["ref_cols"]), cu(rpt), n_cut, out)
    assert np.array_equal(host(out), 2 * d["ref_support"])


def test_segment_isin2_any_acyclic_orientation():
    """Rows oriented by a random total order (not by id) still count every
    triangle once, as the reference's merge does."""
    rows, cols, rp, verts = _rand_graph(5)
    V = len(verts)
    perm = np.random.default_rng(1).permutation(V)
    lo = np.where(perm[rows] < perm[cols], rows, cols)
    hi = np.where(perm[rows] < perm[cols], cols, rows)
    order = np.lexsort((hi, lo))
    r2, c2 = lo[order].astype(np.int32), hi[order].astype(np.int32)
    rp2 = np.concatenate([[0], np.cumsum(np.bincount(r2, minlength=V))]).astype(np.int32)
    ref = O.support(r2, c2, rp2, 1)
    out = torch.zeros(len(c2), dtype=torch.int32, device="cuda")
    tt.segment_isin2(cu(r2), cu(c2), cu(rp2), out)
    assert np.array_equal(host(out), ref)


def _affect_case(seed, n_cut, holes=True):
    rows, cols, rp, verts = _rand_graph(seed)
    V = len(verts)
    rpt = O.tiling_row_ptr(rows, cols, V, n_cut)
    sup = O.support(rows, cols, rpt, n_cut)
    rng = np.random.default_rng(seed + 100)
    E = cols.shape[0]
    cols = cols.copy()
    if holes:  # previously peeled edges carry the -1 sentinel (singlegpu_truss.py:118)
        dead = rng.random(E) < 0.15
        cols[dead] = -1
    else:
        dead = np.zeros(E, bool)
    l = max(1, int(np.percentile(sup, 40)))
    mark = (rng.random(E) < 0.8) & ~dead
    e_aff = np.nonzero((rng.random(E) < 0.6) & ~dead)[0].astype(np.int32)
    return rows, cols, rpt, sup, l, mark.astype(np.uint8), e_aff


def _check_racy(a_sup, a_nm, b_sup, b_nm, l):
    assert np.array_equal(a_nm, b_nm)
    hi = (a_sup > l) | (b_sup > l)
    assert np.array_equal(a_sup[hi], b_sup[hi])
    assert np.all(a_sup[~hi] <= l) and np.all(b_sup[~hi] <= l)


@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("n_cut", [1, 2])
@pytest.mark.parametrize("kind", ["not", "deleted"])
def test_affected_support_ops(seed, n_cut, kind):
    rows, cols, rpt, sup, l, mark, e_aff = _affect_case(seed, n_cut)
    E = cols.shape[0]
    o_sup, o_nm = sup.copy(), np.zeros(E, np.uint8)
    if kind == "not":
        O.all_affected_support_tilenot(e_aff, rows, cols, rpt, n_cut, mark, l, o_nm, o_sup)
    else:
        O.all_affected_support_tile(e_aff, rows, cols, rpt, n_cut, mark, l, o_nm, o_sup)
    g_sup, g_nm = cu(sup), torch.zeros(E, dtype=torch.bool, device="cuda")
    args = (cu(e_aff), cu(rows), cu(cols), cu(rpt))
    m = cu(mark, torch.bool)
    if kind == "not":
        if n_cut == 1:
            tt.sub_AllAffectedSupport_not(*args, m, l, g_nm, g_sup)
        else:
            tt.sub_AllAffectedSupport_tilenot(*args, n_cut, m, l, g_nm, g_sup)
    else:
        if n_cut == 1:
            tt.sub_AllAffectedSupport(*args, m, l, g_nm, g_sup)
        else:
            tt.sub_AllAffectedSupport_tile(*args, n_cut, m, l, g_nm, g_sup)
    _check_racy(host(g_sup), host(g_nm).astype(np.uint8), o_sup, o_nm, l)


@pytest.mark.parametrize("n_cut", [1, 2])
def test_affected_support_windowed(n_cut):
    rows, cols, rpt, sup, l, mark, e_aff = _affect_case(7, n_cut)
    E = cols.shape[0]
    wh = l + 3
    o_sup, o_nm, o_win = sup.copy(), np.zeros(E, np.uint8), np.zeros(E, np.uint8)
    o_buf, o_n = np.zeros(E, np.int32), np.zeros(1, np.int32)
    O.all_affected_support_tilenotwin(e_aff, rows, cols, rpt, n_cut, mark, l, o_nm, o_sup, wh, o_win, o_buf, o_n)
    g_sup, g_nm = cu(sup), torch.zeros(E, dtype=torch.bool, device="cuda")
    g_win = torch.zeros(E, dtype=torch.bool, device="cuda")
    g_buf = torch.zeros(E, dtype=torch.int32, device="cuda")
    g_n = torch.zeros(1, dtype=torch.int32, device="cuda")
    args = (cu(e_aff), cu(rows), cu(cols), cu(rpt))
    m = cu(mark, torch.bool)
    if n_cut == 1:
        tt.sub_AllAffectedSupport_notwin(*args, m, l, g_nm, g_sup, wh, g_win, g_buf, g_n)
    else:
        tt.sub_AllAffectedSupport_tilenotwin(*args, n_cut, m, l, g_nm, g_sup, wh, g_win, g_buf, g_n)
    _check_racy(host(g_sup), host(g_nm).astype(np.uint8), o_sup, o_nm, l)
    assert np.array_equal(host(g_win).astype(np.uint8), o_win)
    n = int(host(g_n)[0])
    assert n == int(o_n[0])
    assert sorted(host(g_buf)[:n].tolist()) == sorted(o_buf[:n].tolist())


@pytest.mark.parametrize("n_cut", [1, 2])
def test_support_k_saturating(n_cut):
    rows, cols, rp, verts = _rand_graph(3)
    rpt = O.tiling_row_ptr(rows, cols, len(verts), n_cut)
    for k in (1, 2, 4, 1000):
        o = np.zeros(cols.shape[0], np.int32)
        O.segment_isin2tile_k(rows, cols, rpt, n_cut, k, o)
        g = torch.zeros(cols.shape[0], dtype=torch.int32, device="cuda")
        if n_cut == 1:
            tt.segment_isin2_k(cu(rows), cu(cols), cu(rpt), k, g)
        else:
            tt.segment_isin2tile_k(cu(rows), cu(cols), cu(rpt), n_cut, k, g)
        assert np.array_equal(np.minimum(host(g), k), np.minimum(o, k))


@pytest.mark.parametrize("n_cut", [1, 2])
def test_sub_affected_support_exact(n_cut):
    rows, cols, rp, verts = _rand_graph(4)
    rpt = O.tiling_row_ptr(rows, cols, len(verts), n_cut)
    sup = O.support(rows, cols, rpt, n_cut)
    mark = (np.random.default_rng(9).random(cols.shape[0]) < 0.2).astype(np.uint8)
    o = sup.copy()
    O.sub_affected_support_tile(rows, cols, rpt, n_cut, mark, o)
    g = cu(sup)
    if n_cut == 1:
        tt.sub_AffectedSupport(cu(rows), cu(cols), cu(rpt), cu(mark, torch.bool), g)
    else:
        tt.sub_AffectedSupport_tile(cu(rows), cu(cols), cu(rpt), n_cut, cu(mark, torch.bool), g)
    assert np.array_equal(host(g), o)


def test_empty_inputs_are_noops():
    z = torch.zeros(0, dtype=torch.int32, device="cuda")
    rp = torch.zeros(1, dtype=torch.int32, device="cuda")
    tt.segment_isin2(z, z, rp, z)
    tt.sub_AllAffectedSupport_not(z, z, z, rp, z.bool(), 1, z.bool(), z)
    tt.segment_add(z, rp, z)


def test_bad_arguments_raise():
    x = torch.zeros(4, dtype=torch.int32, device="cuda")
    with pytest.raises(TypeError):
        tt.segment_isin2(x, x.long(), torch.zeros(5, dtype=torch.int32, device="cuda"), x)
    with pytest.raises(Exception):
        tt.segment_isin2tile(x, x, torch.zeros(4, dtype=torch.int32, device="cuda"), 2, x)  # 4 != V*2+1


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("n_cut,cpu_flow", [(1, False), (2, False), (2, True)])
def test_reference_flow_on_dropin_ops(name, n_cut, cpu_flow):
    """The reference's host-driven k_truss loop run over these operators
    reproduces the reference's peel order exactly."""
    d = GD.load(name)
    V = d["ref_vertices"].shape[0]
    g = CSRCOO(columns=cu(d["ref_cols"]), row_ptr=cu(d["ref_rp_tiled%d" % n_cut]), rows=cu(d["ref_rows"]))
    kmax, et, pt = flow.k_truss(g, n_cut, V, cpu_flow=cpu_flow)
    key = "cpu" if cpu_flow else "sg"
    suffix = "" if cpu_flow else str(n_cut)
    assert kmax == int(d["%s_kmax%s" % (key, suffix)])
    assert np.array_equal(host(et), d["%s_e_truss%s" % (key, suffix)])
    assert np.array_equal(pt.numpy(), d["%s_ptr_truss%s" % (key, suffix)])


def test_reference_flow_with_compaction():
    """Force the compaction branch (singlegpu_truss.py:120-134) on every round."""
    d = GD.load("rmat_s10")
    V = d["ref_vertices"].shape[0]
    g = CSRCOO(columns=cu(d["ref_cols"]), row_ptr=cu(d["ref_rp_tiled2"]), rows=cu(d["ref_rows"]))
    kmax, et, pt = flow.k_truss(g, 2, V, compact_threshold=0)
    assert kmax == int(d["sg_kmax2"])
    assert np.array_equal(host(et), d["sg_e_truss2"])


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("n_cut,skip,compact", [(1, 16, 10000000), (2, 16, 10000000), (2, 3, 10000000), (2, 4, 0)])
def test_windowed_flow_on_dropin_ops(name, n_cut, skip, compact):
    """The support-window flow of multigpu_truss_pre4.py over the *_notwin
    operators: the reference's kmax, per-level peel sets and level offsets
    (the order inside a sub-round follows the concurrently filled window
    buffer); small windows and compaction on every round included."""
    d = GD.load(name)
    V = d["ref_vertices"].shape[0]
    g = CSRCOO(columns=cu(d["ref_cols"]), row_ptr=cu(d["ref_rp_tiled%d" % n_cut]), rows=cu(d["ref_rows"]))
    kmax, et, pt = flow.k_truss_windowed(g, n_cut, V, windows_skip=skip, compact_threshold=compact)
    ref_et, ref_pt = d["sg_e_truss2"], d["sg_ptr_truss2"]
    assert kmax == int(d["sg_kmax2"])
    assert np.array_equal(pt.numpy(), ref_pt)
    et = host(et)
    for j in range(len(ref_pt) - 1):
        a, b = ref_pt[j], ref_pt[j + 1]
        assert np.array_equal(np.sort(et[a:b]), np.sort(ref_et[a:b])), j
