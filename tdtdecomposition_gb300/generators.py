"""Seeded synthetic workloads (edge lists before preprocessing).

They stand in for the SNAP / Network Repository graphs the reference measures
on, which are not available here:

* ``er_edges``       Erdos-Renyi G(n, m): m distinct unordered pairs;
* ``rmat_edges``     R-MAT (a, b, c, d) with 2^scale vertices, m draws;
* ``chung_lu_edges`` power-law expected degrees (exponent gamma, capped);
* ``ba_edges``       Barabasi-Albert preferential attachment (native host code).

Every draw comes from the counter-based stream splitmix64(splitmix64(seed)+j)
(implemented here in numpy and in csrc/gen.cu), so host and device versions
produce the same edges.
"""
import ctypes

import numpy as np

M53 = 1 << 53
_U = np.uint64


def splitmix64(x):
    """Vectorised splitmix64 over uint64 arrays (wrapping arithmetic)."""
    x = np.asarray(x, dtype=_U)
    with np.errstate(over="ignore"):
        x = x + _U(0x9E3779B97F4A7C15)
        x = (x ^ (x >> _U(30))) * _U(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> _U(27))) * _U(0x94D049BB133111EB)
        return x ^ (x >> _U(31))


def stream(seed, start, count):
    key = splitmix64(_U(seed & 0xFFFFFFFFFFFFFFFF))
    with np.errstate(over="ignore"):
        return splitmix64(key + np.arange(start, start + count, dtype=_U))


def er_edges(n, m, seed=0):
    """G(n, m): first m distinct unordered pairs {u != v} of the draw stream
    (u = r0 % n, v = r1 % n per draw)."""
    got = np.zeros((0, 2), np.int64)
    start = 0
    while got.shape[0] < m:
        k = int((m - got.shape[0]) * 1.3) + 64
        r = stream(seed, 2 * start, 2 * k).reshape(k, 2)
        u = (r[:, 0] % _U(n)).astype(np.int64)
        v = (r[:, 1] % _U(n)).astype(np.int64)
        keep = u != v
        pairs = np.stack([np.minimum(u, v), np.maximum(u, v)], 1)[keep]
        allp = np.concatenate([got, pairs])
        _, first = np.unique(allp[:, 0] * n + allp[:, 1], return_index=True)
        got = allp[np.sort(first)]
        start += k
    return got[:m, 0].astype(np.int32), got[:m, 1].astype(np.int32)


def rmat_thresholds(a, b, c):
    return int(a * M53), int((a + b) * M53), int((a + b + c) * M53)


def rmat_edges(scale, m, a=0.57, b=0.19, c=0.19, seed=1):
    """Host R-MAT (same stream as tdt_gen_rmat); for small scales."""
    ta, tab, tabc = (_U(t) for t in rmat_thresholds(a, b, c))
    key = splitmix64(_U(seed))
    src = np.zeros(m, np.uint64)
    dst = np.zeros(m, np.uint64)
    idx = np.arange(m, dtype=_U) * _U(scale)
    with np.errstate(over="ignore"):
        for bit in range(scale):
            r = splitmix64(key + idx + _U(bit)) >> _U(11)
            bs = (r >= tab).astype(_U)
            bd = (((r >= ta) & (r < tab)) | (r >= tabc)).astype(_U)
            src = (src << _U(1)) | bs
            dst = (dst << _U(1)) | bd
    return src.astype(np.int32), dst.astype(np.int32)


def rmat_edges_device(scale, m, a=0.57, b=0.19, c=0.19, seed=1, device="cuda"):
    """R-MAT on the GPU (tdt_gen_rmat); returns int32 CUDA tensors."""
    import torch
    from . import _lib
    L = _lib.load()
    src = torch.empty(m, dtype=torch.int32, device=device)
    dst = torch.empty(m, dtype=torch.int32, device=device)
    ta, tab, tabc = rmat_thresholds(a, b, c)
    fn = L.tdt_gen_rmat
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                   ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    with torch.cuda.device(src.device):
        _lib.check(fn(scale, m, seed, ta, tab, tabc, src.data_ptr(), dst.data_ptr(),
                      torch.cuda.current_stream(src.device).cuda_stream), "tdt_gen_rmat")
    return src, dst


def chung_lu_weights(n, gamma=2.1, mean_degree=40.0, max_degree=1 << 20):
    """Cumulative integer weights (uint64[n]) of chung_lu_edges."""
    i = np.arange(n, dtype=np.float64)
    w = (i + 1.0) ** (-1.0 / (gamma - 1.0))
    w *= mean_degree * n / w.sum()
    w = np.minimum(w, float(max_degree))
    w *= mean_degree * n / w.sum()
    w = np.minimum(w, float(max_degree))
    wi = np.maximum(np.round(w * 1024.0), 1).astype(np.uint64)
    return np.cumsum(wi)


def chung_lu_edges(n, gamma=2.1, mean_degree=40.0, max_degree=1 << 20, seed=2, m=None):
    """Chung-Lu: expected degree w_i = c * (i+1)^(-1/(gamma-1)), capped at
    max_degree, scaled to the mean degree; m = n*mean/2 draws, each endpoint
    drawn with probability proportional to w (integer inverse CDF over
    chung_lu_weights)."""
    cum = chung_lu_weights(n, gamma, mean_degree, max_degree)
    total = int(cum[-1])
    if m is None:
        m = int(n * mean_degree / 2)
    r = stream(seed, 0, 2 * m).reshape(m, 2) % _U(total)
    src = np.searchsorted(cum, r[:, 0], side="right").astype(np.int32)
    dst = np.searchsorted(cum, r[:, 1], side="right").astype(np.int32)
    return src, dst


def chung_lu_edges_device(n, gamma=2.1, mean_degree=40.0, max_degree=1 << 20, seed=2, m=None, device="cuda"):
    """chung_lu_edges on the GPU (tdt_gen_chung_lu): the same edges, as int32
    CUDA tensors."""
    import torch
    from . import _lib
    L = _lib.load()
    cum = chung_lu_weights(n, gamma, mean_degree, max_degree)
    total = int(cum[-1])
    if m is None:
        m = int(n * mean_degree / 2)
    cum_d = torch.from_numpy(cum.view(np.int64)).to(device)
    src = torch.empty(m, dtype=torch.int32, device=device)
    dst = torch.empty(m, dtype=torch.int32, device=device)
    fn = L.tdt_gen_chung_lu
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    with torch.cuda.device(src.device):
        _lib.check(fn(n, m, seed, cum_d.data_ptr(), total, src.data_ptr(), dst.data_ptr(),
                      torch.cuda.current_stream(src.device).cuda_stream), "tdt_gen_chung_lu")
    del cum_d
    return src, dst


def ba_edges(n, m, seed):
    """Barabasi-Albert(n, m) via the native generator (tdt_gen_ba, host code)."""
    from . import _lib
    L = _lib.load()
    fn = L.tdt_gen_ba
    fn.restype = ctypes.c_int64
    fn.argtypes = [ctypes.c_int64, ctypes.c_int32, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_int64]
    total = m + (n - m - 1) * m
    src = np.zeros(total, np.int32)
    dst = np.zeros(total, np.int32)
    k = fn(n, m, seed, src.ctypes.data, dst.ctypes.data, total)
    if k != total:
        raise ValueError("tdt_gen_ba(n=%d, m=%d) failed" % (n, m))
    return src, dst
