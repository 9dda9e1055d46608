"""The continuous-batching server: every request's answer equals the same
request decomposed alone (truss numbers, or the k-truss edge mask), whether
it ran alone or mixed into batches, with and without a binding memory budget."""
import numpy as np
import pytest
import torch

from tdtdecomposition_gb300 import generators as G, serve as S, truss as T
from tdtdecomposition_gb300.preprocess import preprocess_edges

pytestmark = pytest.mark.gpu


def _requests(n=14, seed=11):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        if i % 2:
            s, d = G.ba_edges(int(rng.integers(50, 3000)), int(rng.integers(3, 12)), 500 + i)
        else:
            s, d = G.rmat_edges(int(rng.integers(8, 13)), 16 << int(rng.integers(8, 12)), seed=700 + i)
        q = "decompose" if i % 3 else ("ktruss", int(rng.integers(3, 9)))
        reqs.append(S.Request(i, 0.001 * i, torch.from_numpy(s).pin_memory(), torch.from_numpy(d).pin_memory(), q))
    return reqs


def _alone(r):
    g, _ = preprocess_edges(r.src.cuda(), r.dst.cuda())
    return S.answer_for(r.query, T.truss_decompose(g, lists=False).truss).cpu()


@pytest.mark.parametrize("budget", [150e9, None])
def test_each_result_same_alone_and_in_the_mix(budget):
    reqs = _requests()
    if budget is None:  # budget that admits ~2 requests at a time
        budget = 2.2 * max(r.bytes for r in reqs)
    srv = S.TrussServer(memory_budget=budget)
    out = srv.run(reqs, real_time=True)
    for r in out:
        assert r.answer is not None
        assert torch.equal(r.answer, _alone(r)), r.id
    st = S.latency_stats(out)
    assert st["p99_ms"] >= st["p50_ms"] > 0


def test_search_path_and_small_unions_give_the_same_answers():
    """k-truss queries on graphs past search_min_edges run the fixed-level
    search alone; the rest go into unions of at most max_batch_edges edges,
    smallest first.  Every answer equals the request run alone."""
    reqs = _requests(n=16, seed=5)
    srv = S.TrussServer(search_min_edges=2000, max_batch_edges=30000, max_wait_s=0.0)
    out = srv.run(reqs, real_time=False)
    paths = {r.path for r in out}
    assert "search" in paths and "batch" in paths
    for r in out:
        assert torch.equal(r.answer, _alone(r)), r.id
        if r.path == "search":
            assert S.is_ktruss(r.query) and r.num_edges >= 2000
    by = S.latency_by_class(out)
    assert sum(v["requests"] for v in by.values()) == len(out)


def test_resident_graphs_answer_later_queries():
    """Graphs kept under handles answer later queries without ingest: from
    their cached truss numbers once decomposed (a batch kept them), or by one
    call on the resident CSR (the search path kept them without truss
    numbers); triangle counts on the resident CSR."""
    reqs = _requests(n=8, seed=3)
    for r in reqs:
        r.keep, r.handle = True, "g%d" % r.id
    srv = S.TrussServer(search_min_edges=2000)
    srv.run(reqs, real_time=False)
    assert set(srv.resident) == {r.handle for r in reqs}
    later = []
    for i, r in enumerate(reqs):
        for q in ("decompose", ("ktruss", 3 + i % 4), "triangles"):
            later.append(S.Request(100 + len(later), 0.0, None, None, q, handle=r.handle))
    srv.run(later, real_time=False)
    for q in later:
        base = reqs[int(q.handle[1:])]
        g, _ = preprocess_edges(base.src.cuda(), base.dst.cuda())
        assert q.path == "resident"
        if q.query == "triangles":
            assert int(q.answer[0]) == T.triangle_count(g)
        else:
            assert torch.equal(q.answer, S.answer_for(q.query, T.truss_decompose(g, lists=False).truss).cpu())


def test_resident_budget_evicts_least_recently_used():
    reqs = _requests(n=6, seed=9)
    for r in reqs:
        r.keep, r.handle = True, r.id
    srv = S.TrussServer(resident_budget=1)  # keeps only the most recent graph
    srv.run(reqs, real_time=False)
    assert len(srv.resident) == 1
    gone = next(r.handle for r in reqs if r.handle not in srv.resident)
    with pytest.raises(KeyError):
        srv.run([S.Request(99, 0.0, None, None, "decompose", handle=gone)], real_time=False)


def test_pack_device_is_the_disjoint_union():
    from tdtdecomposition_gb300 import batch as B
    gs = []
    for i in range(5):
        s, d = G.ba_edges(200 + 50 * i, 4, 900 + i)
        g, _ = preprocess_edges(torch.as_tensor(s).cuda(), torch.as_tensor(d).cuda())
        gs.append(g)
    bt = S.pack_device(gs, "cuda")
    res = B.decompose(bt, lists=False)
    for i, g in enumerate(gs):
        assert torch.equal(B.per_graph(bt, res, i), T.truss_decompose(g, lists=False).truss)
