"""Autotuner of the work split and launch shape.

The support and listing kernels give a row to one warp when its out-degree is
at most `warp_cap`, to a whole block (shared-memory staged, pairs spread
evenly over 512 threads) when it is at most `heavy_cap`, and search it in
place beyond that; their wedge walk reads one column per lane or 16-byte
chunks of four (`vec`); the peel reads triangles from per-edge lists or
searches for them (`lists`), on a persistent grid of `peel_grid` half-SM
units (0: the size heuristic).  Which choice is fastest depends on the
degree profile and size of the workload, so the tuner times the candidates
on the workload itself (CUDA events, after one warm-up run each), one
dimension at a time from the defaults (a coordinate search: the split, then
the lists, the peel grid and the walk width), and caches the winner per
workload signature (edge count and out-degree profile, bucketed).  Results
do not depend on any of these choices."""
import math

import torch

from . import _lib, truss as T

CANDIDATES = [(256, 0), (128, 0), (64, 0), (32, 0), (256, 2048)]
PEEL_GRIDS = (0, 1, 2, 4)
VEC_WALK = (1, 0)
_cache = {}


class Config(tuple):
    """(warp_cap, heavy_cap, lists, peel_grid, vec); the first three keep the
    order of the earlier (warp_cap, heavy_cap, lists) result."""

    __slots__ = ()

    def __new__(cls, warp_cap, heavy_cap, lists, peel_grid=0, vec=1):
        return super().__new__(cls, (warp_cap, heavy_cap, lists, peel_grid, vec))

    warp_cap = property(lambda self: self[0])
    heavy_cap = property(lambda self: self[1])
    lists = property(lambda self: self[2])
    peel_grid = property(lambda self: self[3])
    vec = property(lambda self: self[4])


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


def apply(cfg):
    """Set the library knobs of a Config (the lists choice is a call argument)."""
    L = _lib.load()
    L.tdt_set_support_caps(cfg.warp_cap, cfg.heavy_cap)
    L.tdt_set_peel_grid(cfg.peel_grid)
    L.tdt_set_vector_walk(cfg.vec)


def tune(graph, workspace=None, lists_options=(True, False), candidates=CANDIDATES, peel_grids=PEEL_GRIDS,
         vec_options=VEC_WALK, verbose=False):
    """Returns the Config for this workload and applies its knobs; cached per
    signature."""
    key = signature(graph)
    if key in _cache:
        apply(_cache[key])
        return _cache[key]
    timed = {}

    def cost(cfg):
        if cfg not in timed:
            apply(cfg)
            T.truss_decompose(graph, workspace=workspace, lists=cfg.lists, sync=True)  # warm-up
            timed[cfg] = _time(lambda: T.truss_decompose(graph, workspace=workspace, lists=cfg.lists, sync=False))
            if verbose:
                print("autotune", key, tuple(cfg), "%.2f ms" % timed[cfg])
        return timed[cfg]

    best = Config(candidates[0][0], candidates[0][1], lists_options[0], peel_grids[0], vec_options[0])
    dims = [
        [Config(wc, hc, best.lists, best.peel_grid, best.vec) for wc, hc in candidates],
        None, None, None,
    ]
    for d in range(4):
        if d == 0:
            opts = dims[0]
        elif d == 1:
            opts = [Config(best.warp_cap, best.heavy_cap, li, best.peel_grid, best.vec) for li in lists_options]
        elif d == 2:
            opts = [Config(best.warp_cap, best.heavy_cap, best.lists, pg, best.vec) for pg in peel_grids]
        else:
            opts = [Config(best.warp_cap, best.heavy_cap, best.lists, best.peel_grid, v) for v in vec_options]
        best = min(opts, key=cost)
    _cache[key] = best
    apply(best)
    return best


def reset():
    _cache.clear()
    apply(Config(0, 0, True, 0, 1))
