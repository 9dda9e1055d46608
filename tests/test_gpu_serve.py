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
