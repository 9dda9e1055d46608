"""The oracle pinned against the reference's own outputs (tests/golden, made
by tests/golden/make_golden.py from the reference code) and against
networkx.  CPU only."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import _golden as GD

CASES = GD.names()


@pytest.mark.parametrize("name", CASES)
def test_preprocessing_matches_reference(name):
    d = GD.load(name)
    rows, cols, rp, verts = O.preprocess(d["pairs"], stable=False)
    assert np.array_equal(rows, d["ref_rows"])
    assert np.array_equal(cols, d["ref_cols"])
    assert np.array_equal(rp, d["ref_rp"])
    assert np.array_equal(verts, d["ref_vertices"])
    for n_cut in (1, 2):
        assert np.array_equal(O.tiling_row_ptr(rows, cols, len(verts), n_cut), d["ref_rp_tiled%d" % n_cut])


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("n_cut", [1, 2, 3])
def test_support_matches_reference(name, n_cut):
    d = GD.load(name)
    V = d["ref_vertices"].shape[0]
    rpt = O.tiling_row_ptr(d["ref_rows"], d["ref_cols"], V, n_cut)
    assert np.array_equal(O.support(d["ref_rows"], d["ref_cols"], rpt, n_cut), d["ref_support"])


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("n_cut", [1, 2])
def test_k_truss_matches_reference_driver(name, n_cut):
    d = GD.load(name)
    V = d["ref_vertices"].shape[0]
    kmax, et, pt, _ = O.k_truss(d["ref_rows"], d["ref_cols"], d["ref_rp_tiled%d" % n_cut], V, n_cut)
    assert kmax == int(d["sg_kmax%d" % n_cut])
    assert np.array_equal(et, d["sg_e_truss%d" % n_cut])
    assert np.array_equal(pt, d["sg_ptr_truss%d" % n_cut])


@pytest.mark.parametrize("name", CASES)
def test_cpu_flow_matches_reference_cpu_path(name):
    d = GD.load(name)
    V = d["ref_vertices"].shape[0]
    kmax, et, pt, _ = O.k_truss(d["ref_rows"], d["ref_cols"], d["ref_rp_tiled2"], V, 2, cpu_flow=True)
    assert kmax == int(d["cpu_kmax"])
    assert np.array_equal(et, d["cpu_e_truss"])
    assert np.array_equal(pt, d["cpu_ptr_truss"])
    # both reference flows produce the same peel order
    assert np.array_equal(d["cpu_e_truss"], d["sg_e_truss2"])


@pytest.mark.parametrize("name", CASES)
def test_ktruss_search_matches_reference_driver(name):
    d = GD.load(name)
    V = d["ref_vertices"].shape[0]
    for k in d["kt_ks"]:
        r, c = O.ktruss_search(d["ref_rows"], d["ref_cols"], d["ref_rp_tiled2"], V, 2, int(k))
        assert GD.edge_set(r, c) == GD.edge_set(d["kt_rows_k%d" % k], d["kt_cols_k%d" % k]), k


@pytest.mark.parametrize("name", [n for n in CASES if n != "er_4096_65536"])
def test_truss_numbers_match_networkx(name):
    d = GD.load(name)
    truss = GD.truss_from_levels(d["sg_e_truss2"], d["sg_ptr_truss2"], d["ref_cols"].shape[0])
    m = O.undirected_truss_map(d["ref_rows"], d["ref_cols"], truss, d["ref_vertices"])
    nx = {(int(a), int(b)): int(t) for (a, b), t in zip(d["nx_pairs"], d["nx_truss"])}
    assert m == nx


@pytest.mark.parametrize("name", CASES)
def test_stable_rank_gives_same_truss_numbers(name):
    """Truss numbers are orientation-invariant: the (degree, id) rank and the
    reference's numpy tie order agree on every undirected edge."""
    d = GD.load(name)
    rows, cols, rp, verts = O.preprocess(d["pairs"], stable=True)
    _, _, _, truss = O.k_truss(rows, cols, O.tiling_row_ptr(rows, cols, len(verts), 2), len(verts), 2)
    ref_truss = GD.truss_from_levels(d["sg_e_truss2"], d["sg_ptr_truss2"], d["ref_cols"].shape[0])
    a = O.undirected_truss_map(rows, cols, truss, verts)
    b = O.undirected_truss_map(d["ref_rows"], d["ref_cols"], ref_truss, d["ref_vertices"])
    assert a == b


def test_fixture_known_answers():
    """test_data/example_graph.txt: 27 edges, 24 triangles, kmax 5; k-truss
    sizes 27 / 24 / 10 for k = 3 / 4 / 5."""
    d = GD.load("fixture")
    assert d["ref_cols"].shape[0] == 27
    assert int(d["ref_support"].sum()) // 3 == 24
    assert int(d["sg_kmax2"]) == 5
    sizes = {int(k): len(d["kt_rows_k%d" % k]) for k in d["kt_ks"]}
    assert sizes[3] == 27 and sizes[4] == 24 and sizes[5] == 10


def _ref_or_skip():
    R = O.ref_ops()
    if R is None:
        pytest.skip("reference operators (oracle/_ref) not built here")
    return R


def _random_oriented(seed, V=300, m=3000):
    rng = np.random.default_rng(seed)
    u = rng.integers(0, V, m)
    v = rng.integers(0, V, m)
    pairs = np.stack([u, v], 1).astype(np.int32)
    return O.preprocess(pairs, stable=True)


@pytest.mark.parametrize("seed", [0, 1])
def test_affected_ops_match_reference_operator(seed):
    """The restated peel update (deleted-mark semantics) against the
    reference's own OpenMP operator: n_mark and supports above l agree."""
    R = _ref_or_skip()
    rows, cols, rp, verts = _random_oriented(seed)
    V = len(verts)
    rpt = O.tiling_row_ptr(rows, cols, V, 2)
    sup = O.support(rows, cols, rpt, 2)
    l = max(1, int(np.median(sup)))
    rng = np.random.default_rng(seed + 10)
    mark = (rng.random(cols.shape[0]) < 0.1).astype(np.uint8)
    e_aff = np.nonzero(rng.random(cols.shape[0]) < 0.5)[0].astype(np.int32)
    a_sup, a_nm = sup.copy(), np.zeros(cols.shape[0], np.uint8)
    b_sup, b_nm = sup.copy(), np.zeros(cols.shape[0], np.uint8)
    O.all_affected_support_tile(e_aff, rows, cols, rpt, 2, mark, l, a_nm, a_sup)
    R.ref_all_affected_support_tile(e_aff, rows, cols, rpt, 2, mark, l, b_nm, b_sup, e_aff.shape[0] * 2)
    assert np.array_equal(a_nm, b_nm)
    hi = (a_sup > l) | (b_sup > l)
    assert np.array_equal(a_sup[hi], b_sup[hi])
