"""Whole-path API: truss decomposition, k-truss search and triangle count on
one GB300, through the C ABI (tdt_truss_decompose / tdt_ktruss_search /
tdt_triangle_count).

Inputs are the oriented CSRCOO (rows < columns, columns sorted within a row)
with untiled row offsets; results are keyed by CSR edge position, like the
reference's e_truss (singlegpu_truss.py:83-101 keeps original positions in
``edges``).
"""
import ctypes
from typing import NamedTuple

import torch

from . import _lib

STAT_STATUS, STAT_KMAX, STAT_NPTR, STAT_ROUNDS, STAT_TRIANGLES, STAT_NETRUSS, STAT_ALIVE, STAT_LISTED = range(8)
STAT_COUNT = 8


class TrussResult(NamedTuple):
    truss: torch.Tensor       # int32[E]: truss number per edge (2 = in no triangle)
    e_truss: torch.Tensor     # int32[n]: the reference's peel order (support-0 edges excluded)
    ptr_truss: torch.Tensor   # int32[kmax-1]: per-level offsets into e_truss
    kmax: int
    triangles: int
    rounds: int
    listed: bool = False      # the peel read per-edge triangle lists (else it searched)
    listing: int = 0          # 0 search peel; lists written by 1 a second walk, 2 the one walk


class Workspace:
    """Device scratch reused across calls (grown on demand, torch-allocated).

    It also remembers the triangle count of the graphs it has served, so that
    later calls on the same graph can size the per-edge triangle lists."""

    def __init__(self, device=None):
        self.device = torch.device(device) if device is not None else torch.device("cuda")
        self.buf = None
        self.triangles = {}

    def get(self, nbytes):
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = None
            self.buf = torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=self.device)
        return self.buf


def _graph_key(cols, rp):
    return (cols.data_ptr(), cols.shape[0], rp.shape[0])


LIST_BUDGET_FRACTION = 0.6
# lists plus the one walk's staging area (which is dead memory once the lists
# are packed) may take more of the free memory
STAGE_BUDGET_FRACTION = 0.75


def stage_bytes(cols, rp, rows=None):
    """Bytes of the one-walk pass's staging area: 8 per slot of the role-A /
    role-B bounds of every edge e = (u, v) at position i of row u:
    min(d+(u) - i - 1, d+(v)) + min(i, d-(v) - 1), the bounds the device
    computes (stage_bounds_kernel)."""
    rp = rp.to(torch.int64)
    V, E = rp.shape[0] - 1, cols.shape[0]
    if E == 0:
        return 0
    dplus = rp[1:] - rp[:-1]
    if rows is None:
        rows = torch.repeat_interleave(torch.arange(V, device=cols.device), dplus)
    u = rows.to(torch.int64)
    v = cols.to(torch.int64)
    i = torch.arange(E, device=cols.device) - rp[u]
    indeg = torch.bincount(v, minlength=V)
    a = torch.minimum(dplus[u] - i - 1, dplus[v]).clamp_min_(0)
    b = torch.minimum(i, indeg[v] - 1).clamp_min_(0)
    return 8 * int((a + b).sum())


def _list_bytes(ws, cols, rp, lists, base, rows=None):
    """Bytes for the workspace's list tail, or 0 to let the peel search the
    adjacency instead: the per-edge triangle lists (24 bytes per triangle)
    plus, when that fits too, the staging area of the one-walk pass (which
    then counts and lists in one walk instead of two).  lists:
    True/False/"auto" ("auto" keeps lists whenever they fit: the listed peel
    is the faster one at every size, from 10 K edges up)."""
    if lists is False:
        return 0
    key = _graph_key(cols, rp)
    T = ws.triangles.get(key)
    if T is None:
        T = triangle_count_arrays(cols, rp, ws)
        ws.triangles[key] = T
    sk = ("stage",) + key
    S = ws.triangles.get(sk)
    if S is None:
        S = stage_bytes(cols, rp, rows)
        ws.triangles[sk] = S
    need = 24 * T + 256
    if lists is True:
        return need + S
    free, _ = torch.cuda.mem_get_info(cols.device)
    have = free + (ws.buf.numel() if ws.buf is not None else 0) - base
    if need + S <= STAGE_BUDGET_FRACTION * have:
        return need + S
    return need if need <= LIST_BUDGET_FRACTION * have else 0


_default_ws = {}


def _ws_for(device, ws):
    if ws is not None:
        return ws
    key = torch.device(device).index if torch.device(device).index is not None else torch.cuda.current_device()
    if key not in _default_ws:
        _default_ws[key] = Workspace(torch.device("cuda", key))
    return _default_ws[key]


def _graph_arrays(graph):
    cols, rp, rows = graph.columns, graph.row_ptr, graph.rows
    if not cols.is_cuda:
        raise TypeError("graph must be on a CUDA device (no CPU path)")
    if cols.dtype != torch.int32 or not cols.is_contiguous():
        raise TypeError("columns must be contiguous int32")
    if rows is not None and (rows.dtype != torch.int32 or not rows.is_contiguous()):
        raise TypeError("rows must be contiguous int32")
    if rp.shape[0] < 1:
        raise ValueError("row_ptr must have V+1 entries")
    if rp.dtype != torch.int64:
        rp = rp.to(torch.int64)
    rp = rp.contiguous()
    return rows, cols, rp


def _check_stats(stats_host, where):
    st = int(stats_host[STAT_STATUS])
    if st != 0:
        raise _lib.TdtError(st, where, "reported by the device")


def truss_decompose(graph, workspace=None, stream=None, sync=True, lists="auto", list_budget=None):
    """Full truss decomposition (singlegpu_truss.py:67-158 + :38-45).

    lists: "auto" keeps per-edge triangle lists in the workspace when they fit
    in LIST_BUDGET_FRACTION of the free device memory (the first call on a
    graph then counts its triangles first), True always, False never.
    list_budget (bytes): instead, give the lists a fixed workspace tail and
    let the device decide (lists when 24 T bytes fit, else the search peel),
    with no counting pass."""
    L = _lib.load()
    rows, cols, rp = _graph_arrays(graph)
    dev = cols.device
    V, E = rp.shape[0] - 1, cols.shape[0]
    truss = torch.empty(E, dtype=torch.int32, device=dev)
    e_truss = torch.empty(max(E, 1), dtype=torch.int32, device=dev)
    cap = E + 2
    ptr = torch.empty(cap, dtype=torch.int32, device=dev)
    stats = torch.zeros(STAT_COUNT, dtype=torch.int64, device=dev)
    need = L.tdt_decompose_workspace_bytes(V, E)
    wso = _ws_for(dev, workspace)
    base = (need + 255) // 256 * 256
    tail = int(list_budget) if list_budget is not None else _list_bytes(wso, cols, rp, lists, base, rows)
    ws = wso.get(base + tail)
    s = (stream or torch.cuda.current_stream(dev)).cuda_stream
    # pass the requested size, not the (possibly larger, shared) buffer: the
    # device keeps lists exactly when the tail it is given holds them
    with torch.cuda.device(cols.device):
        rc = L.tdt_truss_decompose(rows.data_ptr() if rows is not None else None, cols.data_ptr(), rp.data_ptr(), V, E,
                                   truss.data_ptr(), e_truss.data_ptr(), ptr.data_ptr(), cap, stats.data_ptr(),
                                   ws.data_ptr(), base + tail, s)
    _lib.check(rc, "tdt_truss_decompose")
    if not sync:
        return truss, e_truss, ptr, stats
    sh = stats.cpu()
    _check_stats(sh, "tdt_truss_decompose")
    return TrussResult(truss, e_truss[: int(sh[STAT_NETRUSS])], ptr[: int(sh[STAT_NPTR])], int(sh[STAT_KMAX]),
                       int(sh[STAT_TRIANGLES]), int(sh[STAT_ROUNDS]), bool(sh[STAT_LISTED]), int(sh[STAT_LISTED]))


def ktruss_search(graph, k, workspace=None, stream=None, lists="auto"):
    """Edges of the k-truss (ktruss_search/ktruss_cuda.py:383-463 with l=k-2):
    returns a bool mask over the CSR edge positions."""
    L = _lib.load()
    rows, cols, rp = _graph_arrays(graph)
    dev = cols.device
    V, E = rp.shape[0] - 1, cols.shape[0]
    mask = torch.empty(E, dtype=torch.bool, device=dev)
    stats = torch.zeros(STAT_COUNT, dtype=torch.int64, device=dev)
    wso = _ws_for(dev, workspace)
    base = (L.tdt_decompose_workspace_bytes(V, E) + 255) // 256 * 256
    tail = _list_bytes(wso, cols, rp, lists, base, rows)
    ws = wso.get(base + tail)
    s = (stream or torch.cuda.current_stream(dev)).cuda_stream
    with torch.cuda.device(cols.device):
        rc = L.tdt_ktruss_search(rows.data_ptr() if rows is not None else None, cols.data_ptr(), rp.data_ptr(), V, E,
                                 int(k), mask.data_ptr(), stats.data_ptr(), ws.data_ptr(), base + tail, s)
    _lib.check(rc, "tdt_ktruss_search")
    _check_stats(stats.cpu(), "tdt_ktruss_search")
    return mask


def triangle_count_arrays(cols, rp, ws):
    L = _lib.load()
    V, E = rp.shape[0] - 1, cols.shape[0]
    stats = torch.zeros(STAT_COUNT, dtype=torch.int64, device=cols.device)
    buf = ws.get(L.tdt_decompose_workspace_bytes(V, E))
    with torch.cuda.device(cols.device):
        rc = L.tdt_triangle_count(cols.data_ptr(), rp.data_ptr(), V, E, None, stats.data_ptr(), buf.data_ptr(),
                                  buf.numel(), torch.cuda.current_stream(cols.device).cuda_stream)
    _lib.check(rc, "tdt_triangle_count")
    sh = stats.cpu()
    _check_stats(sh, "tdt_triangle_count")
    return int(sh[STAT_TRIANGLES])


def triangle_count(graph, workspace=None, stream=None, return_support=False):
    """Triangle count = sum(support) / 3; optionally the per-edge support."""
    L = _lib.load()
    _, cols, rp = _graph_arrays(graph)
    dev = cols.device
    V, E = rp.shape[0] - 1, cols.shape[0]
    support = torch.empty(E, dtype=torch.int32, device=dev) if return_support else None
    stats = torch.zeros(STAT_COUNT, dtype=torch.int64, device=dev)
    ws = _ws_for(dev, workspace).get(L.tdt_decompose_workspace_bytes(V, E))
    s = (stream or torch.cuda.current_stream(dev)).cuda_stream
    with torch.cuda.device(cols.device):
        rc = L.tdt_triangle_count(cols.data_ptr(), rp.data_ptr(), V, E,
                                  support.data_ptr() if support is not None else None,
                                  stats.data_ptr(), ws.data_ptr(), ws.numel(), s)
    _lib.check(rc, "tdt_triangle_count")
    sh = stats.cpu()
    _check_stats(sh, "tdt_triangle_count")
    T = int(sh[STAT_TRIANGLES])
    return (T, support) if return_support else T


PHASES = ("support", "listing", "peel", "outputs")


class PhaseProfile:
    """Phase times of the whole-path calls made inside a ``with`` block,
    from CUDA events recorded on their streams (tdt_profile_start /
    tdt_profile_stop): ``ms[phase]`` summed over the calls, ``calls`` the
    number recorded.  The reference prints host-clock times of its support
    and peel phases (singlegpu_truss.py:69-77, :153-157)."""

    def __init__(self, max_calls=4096):
        self.max_calls = int(max_calls)
        self.ms = None
        self.calls = 0

    def __enter__(self):
        _lib.check(_lib.load().tdt_profile_start(self.max_calls), "tdt_profile_start")
        return self

    def __exit__(self, exc_type, exc, tb):
        ph = (ctypes.c_float * 4)()
        n = ctypes.c_int()
        rc = _lib.load().tdt_profile_stop(ph, ctypes.byref(n))
        if exc_type is None:
            _lib.check(rc, "tdt_profile_stop")
        self.ms = dict(zip(PHASES, (float(x) for x in ph)))
        self.calls = n.value
        return False


def peel_clock(workspace, stream=None):
    """Block 0's clock (ms) of the last peel run in `workspace`: candidate
    processing, grid-barrier waits, level changes and the whole kernel."""
    if workspace is None or workspace.buf is None:
        raise ValueError("peel_clock needs the Workspace the decomposition ran in")
    ns = (ctypes.c_longlong * 4)()
    s = (stream or torch.cuda.current_stream(workspace.buf.device)).cuda_stream
    with torch.cuda.device(workspace.buf.device):
        _lib.check(_lib.load().tdt_peel_clock(workspace.buf.data_ptr(), ns, s), "tdt_peel_clock")
    return dict(zip(("processing", "barrier_waits", "level_changes", "total"), (x / 1e6 for x in ns)))
