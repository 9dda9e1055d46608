"""Seeded workloads of the benchmark configurations (synthetic stand-ins for
the SNAP / Network Repository graphs, which are not available here).

* batch of Barabasi-Albert graphs: G graphs, n log-uniform in [64, 16384],
  attachment m uniform in {4..16}, graph i seeded 1000 + i;
* single R-MAT graph: scale, edge factor 16, (a,b,c,d) = (.57,.19,.19,.05);
* served request stream: Poisson arrivals, each request a seeded graph (half
  Barabasi-Albert with n log-uniform in [256, 2^18] and m in {4..16}, half
  R-MAT with scale uniform in 12..20, edge factor 16) asking for a full
  decomposition or a k-truss search with k uniform in [3, 20].
"""
import numpy as np

from . import generators as G


def ba_batch_params(num_graphs=4096, seed=1000, n_lo=64, n_hi=16384):
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(n_lo), np.log(n_hi), num_graphs)).round().astype(np.int64)
    m = rng.integers(4, 17, num_graphs)
    n = np.maximum(n, m + 2)
    return n, m


def ba_batch_edges(num_graphs=4096, seed=1000):
    """Concatenated raw edge lists of the batch: (src, dst, vertex_group),
    graph i's vertex ids shifted past graph i-1's."""
    n, m = ba_batch_params(num_graphs, seed)
    srcs, dsts = [], []
    off = 0
    for i in range(num_graphs):
        s, d = G.ba_edges(int(n[i]), int(m[i]), seed + i)
        srcs.append(s + off)
        dsts.append(d + off)
        off += int(n[i])
    vgroup = np.repeat(np.arange(num_graphs, dtype=np.int32), n)
    return np.concatenate(srcs), np.concatenate(dsts), vgroup


def request_stream(num_requests, rate_per_s, seed=7, ba_n=(256, 1 << 18), rmat_scales=(12, 20)):
    """Poisson request stream: list of dicts with arrival time (s), kind
    ('ba'/'rmat'), generator parameters, query ('decompose' or ('ktruss', k))."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate_per_s, num_requests))
    reqs = []
    for i in range(num_requests):
        if rng.random() < 0.5:
            n = int(round(np.exp(rng.uniform(np.log(ba_n[0]), np.log(ba_n[1])))))
            gen = {"kind": "ba", "n": n, "m": int(rng.integers(4, 17)), "seed": 50000 + i}
        else:
            gen = {"kind": "rmat", "scale": int(rng.integers(rmat_scales[0], rmat_scales[1] + 1)), "seed": 90000 + i}
        q = "decompose" if rng.random() < 0.5 else ("ktruss", int(rng.integers(3, 21)))
        reqs.append({"id": i, "arrival": float(t[i]), "gen": gen, "query": q})
    return reqs
