"""Host-side logic that needs no GPU: generators, argument checks of the
drop-in operators, the CSRCOO container, the server's ingest grouping."""
import numpy as np
import pytest
import torch

from tdtdecomposition_gb300 import CSRCOO, generators as G, tiling_row_ptr, trusstensor as tt
from oracle import oracle as O


def test_splitmix_stream_is_deterministic():
    a = G.stream(7, 0, 100)
    b = G.stream(7, 0, 100)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, G.stream(8, 0, 100))
    assert np.array_equal(G.stream(7, 50, 50), a[50:])


def test_er_has_m_distinct_pairs():
    s, d = G.er_edges(256, 2000, seed=3)
    assert len(s) == 2000
    assert np.all(s < d)
    assert len(set(zip(s.tolist(), d.tolist()))) == 2000


def test_rmat_bits_and_skew():
    s, d = G.rmat_edges(12, 1 << 15, seed=1)
    assert s.min() >= 0 and s.max() < 4096 and d.max() < 4096
    deg = np.bincount(np.concatenate([s, d]), minlength=4096)
    assert deg.max() > 20 * max(1.0, deg.mean())  # skewed


def test_ba_generator_deterministic_and_sized():
    s, d = G.ba_edges(500, 6, seed=1001)
    s2, d2 = G.ba_edges(500, 6, seed=1001)
    assert np.array_equal(s, s2) and np.array_equal(d, d2)
    assert len(s) == 6 + (500 - 7) * 6
    rows, cols, rp, verts = O.preprocess(np.stack([s, d], 1))
    assert len(cols) == len(s)  # BA draws distinct targets: no duplicates


def test_chung_lu_degree_cap():
    s, d = G.chung_lu_edges(2000, gamma=2.1, mean_degree=10, max_degree=64, seed=2)
    deg = np.bincount(np.concatenate([s, d]))
    assert deg.max() < 64 * 1.6


def test_tiling_row_ptr_matches_oracle():
    rows, cols, rp, verts = O.preprocess(np.stack(G.rmat_edges(9, 5000, seed=4), 1))
    g = CSRCOO.from_numpy(rows, cols, rp)
    for n_cut in (1, 2, 3):
        assert np.array_equal(tiling_row_ptr(g, n_cut).numpy(), O.tiling_row_ptr(rows, cols, len(verts), n_cut))


def test_operators_reject_cpu_tensors():
    x = torch.zeros(4, dtype=torch.int32)
    with pytest.raises(TypeError):
        tt.segment_add(x, torch.zeros(5, dtype=torch.int32), x)
    with pytest.raises(TypeError):
        tt.segment_isin2tile(x, x, torch.zeros(5, dtype=torch.int32), 2, x)


def test_research_operators_check_their_arguments():
    """The research-variant operators are real: CPU tensors are refused like
    every other operator's (there is no CPU path)."""
    x = torch.zeros(4, dtype=torch.int32)
    b = torch.zeros(4, dtype=torch.bool)
    with pytest.raises(TypeError):
        tt.peeling_direct_oo(x, x, x, x, x, b, b, b, 1)
    with pytest.raises(TypeError):
        tt.segment_isinis_m(x, x, x, x, b, b)
    assert all(not getattr(tt, n).__doc__ is None for n in tt.__all__)
    assert len([n for n in tt.__all__ if not n.endswith("_k") and "AffectedSupport" not in n
                or n.startswith("sub_AllAffected")]) >= 20


def test_server_ingest_groups_are_capped():
    """The server's ingest takes what is queued up to a draw cap, so a burst
    is split into groups and the first decomposition starts early."""
    import queue
    from tdtdecomposition_gb300 import serve as S

    def req(i, n):
        return S.Request(i, 0.0, torch.zeros(n, dtype=torch.int32), torch.zeros(n, dtype=torch.int32), "decompose")

    q = queue.Queue()
    for i in range(4):
        q.put(req(i, 3))
    q.put(None)
    g, stop = S.take_group(q, 8)          # 3 + 3 < 8, the third reaches 9
    assert [r.id for r in g] == [0, 1, 2] and not stop
    g, stop = S.take_group(q, 8)          # the last request, then the end of the stream
    assert [r.id for r in g] == [3] and stop

    q.put(req(7, 20))
    q.put(req(8, 1))
    g, stop = S.take_group(q, 8)          # one request above the cap goes alone
    assert [r.id for r in g] == [7] and not stop
    g, stop = S.take_group(q, 8)          # nothing else queued: no wait for more
    assert [r.id for r in g] == [8] and not stop

    q.put(None)
    assert S.take_group(q, 8) == ([], True)


def test_server_ingests_search_candidates_alone():
    """A request the server may answer by the fixed-level search (a k-truss
    query on a large edge list) forms an ingest group of its own; one met in
    the middle of a group is carried to the next."""
    import queue
    from tdtdecomposition_gb300 import serve as S

    def req(i, n, q="decompose"):
        return S.Request(i, 0.0, torch.zeros(n, dtype=torch.int32), torch.zeros(n, dtype=torch.int32), q)

    alone = lambda r: S.is_ktruss(r.query) and len(r.src) >= 5  # noqa: E731
    q, carry = queue.Queue(), []
    for r in (req(0, 2), req(1, 6, ("ktruss", 4)), req(2, 2), req(3, 2, ("ktruss", 3)), req(4, 9, ("ktruss", 5))):
        q.put(r)
    q.put(None)
    groups = []
    stop = False
    while not stop:
        g, stop = S.take_group(q, 100, alone, carry)
        groups.append([r.id for r in g])
    assert groups == [[0], [1], [2, 3], [4], []]
