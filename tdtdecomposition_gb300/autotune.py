"""Autotuner of the work split.

The support and listing kernels give a row to one warp when its out-degree is
at most `warp_cap`, to a whole block (shared-memory staged, pairs spread
evenly over 512 threads) when it is at most `heavy_cap`, and search it in
place beyond that; the peel reads triangles from per-edge lists or searches
for them.  Which split is fastest depends on the degree profile of the
workload, so the tuner times the candidates on the workload itself (CUDA
events, after one warm-up run each) and caches the winner per workload
signature (edge count and out-degree profile, bucketed)."""
import math

import torch

from . import _lib, truss as T

CANDIDATES = [(256, 0), (128, 0), (64, 0), (32, 0), (256, 2048)]
_cache = {}


def signature(graph):
    rp = graph.row_ptr.to(torch.int64)
    dp = (rp[1:] - rp[:-1]).float()
    E = graph.num_edges
    return (int(math.log2(max(E, 1))), int(math.log2(float(dp.max()) + 1)),
            int(4 * float(dp.mean()) if dp.numel() else 0))


def _time(fn, reps=1):
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def tune(graph, workspace=None, lists_options=(True, False), candidates=CANDIDATES, verbose=False):
    """Returns (warp_cap, heavy_cap, lists) for this workload and applies the
    caps; cached per signature."""
    L = _lib.load()
    key = signature(graph)
    if key in _cache:
        wc, hc, li = _cache[key]
        L.tdt_set_support_caps(wc, hc)
        return _cache[key]
    best = None
    for lists in lists_options:
        for wc, hc in candidates:
            L.tdt_set_support_caps(wc, hc)
            T.truss_decompose(graph, workspace=workspace, lists=lists, sync=True)  # warm-up
            ms = _time(lambda: T.truss_decompose(graph, workspace=workspace, lists=lists, sync=False))
            if verbose:
                print("autotune", key, (wc, hc, lists), "%.2f ms" % ms)
            if best is None or ms < best[0]:
                best = (ms, (wc, hc, lists))
    _cache[key] = best[1]
    L.tdt_set_support_caps(best[1][0], best[1][1])
    return best[1]


def reset():
    _cache.clear()
    _lib.load().tdt_set_support_caps(0, 0)
