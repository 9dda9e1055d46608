"""Batched truss decomposition of many graphs in one device-resident run.

A batch of oriented graphs whose vertex ranges (and so edge ranges) are
disjoint and increasing is itself one oriented CSR: the disjoint union.  Truss
numbers are properties of each connected component, and every sub-round of
the union peels, in each graph, exactly the edges that graph's own run would
peel in its sub-round of the same level.  So one tdt_truss_decompose call over
the union decomposes every graph of the batch: one support launch, one
listing launch and ONE persistent cooperative peel launch for thousands of
graphs of uneven size (the plain path runs those launches, plus a host sync,
per graph).  Per-graph results are slices of the union's: truss[eb[g]:eb[g+1]]
and kmax[g] = max of that slice.
"""
from typing import List, NamedTuple

import numpy as np
import torch

from . import truss as T
from .graph import CSRCOO


class GraphBatch(NamedTuple):
    graph: CSRCOO              # the disjoint union (int64 row_ptr)
    vertex_offsets: torch.Tensor  # int64[G+1] (host)
    edge_offsets: torch.Tensor    # int64[G+1] (host)

    @property
    def num_graphs(self):
        return self.edge_offsets.numel() - 1


class BatchResult(NamedTuple):
    truss: torch.Tensor        # int32[E_total], graph g owns [edge_offsets[g], edge_offsets[g+1])
    kmax: torch.Tensor         # int64[G] (device)
    union: T.TrussResult


def pack_host(graphs, device="cuda", pin=True):
    """graphs: list of (rows, cols, row_ptr) numpy arrays of oriented graphs
    (local vertex ids).  Packs them on the host into one union (vertex ids of
    graph g shifted by its vertex offset) and copies it to the device in three
    transfers."""
    G = len(graphs)
    vo = np.zeros(G + 1, np.int64)
    eo = np.zeros(G + 1, np.int64)
    for g, (r, c, rp) in enumerate(graphs):
        vo[g + 1] = vo[g] + (len(rp) - 1)
        eo[g + 1] = eo[g] + len(c)
    rows = np.empty(eo[-1], np.int32)
    cols = np.empty(eo[-1], np.int32)
    rpu = np.empty(vo[-1] + 1, np.int64)
    for g, (r, c, rp) in enumerate(graphs):
        rows[eo[g]:eo[g + 1]] = np.asarray(r) + vo[g]
        cols[eo[g]:eo[g + 1]] = np.asarray(c) + vo[g]
        rpu[vo[g]:vo[g + 1]] = np.asarray(rp[:-1], np.int64) + eo[g]
    rpu[-1] = eo[-1]
    ts = [torch.from_numpy(x) for x in (rows, cols, rpu)]
    if pin:
        ts = [t.pin_memory() for t in ts]
    rows_d, cols_d, rp_d = (t.to(device, non_blocking=True) for t in ts)
    return GraphBatch(CSRCOO(columns=cols_d, row_ptr=rp_d, rows=rows_d), torch.from_numpy(vo),
                      torch.from_numpy(eo))


def batch_from_union(graph, edge_offsets, vertex_offsets):
    """Wrap an already packed union (e.g. preprocessed on the device with
    vertex groups) as a GraphBatch."""
    return GraphBatch(graph, torch.as_tensor(vertex_offsets, dtype=torch.int64).cpu(),
                      torch.as_tensor(edge_offsets, dtype=torch.int64).cpu())


def decompose(batch, workspace=None, lists="auto", sync=True, list_budget=None):
    """Decompose every graph of the batch in one device-resident run."""
    res = T.truss_decompose(batch.graph, workspace=workspace, lists=lists, sync=sync, list_budget=list_budget)
    tr = res.truss if sync else res[0]
    eo = batch.edge_offsets.to(tr.device)
    G = batch.num_graphs
    seg = torch.repeat_interleave(torch.arange(G, device=tr.device), eo[1:] - eo[:-1])
    kmax = torch.full((G,), 2, dtype=torch.int64, device=tr.device)
    kmax.scatter_reduce_(0, seg, tr.to(torch.int64), reduce="amax", include_self=True)
    return BatchResult(tr, kmax, res)


def per_graph(batch: GraphBatch, result: BatchResult, g: int):
    """Truss numbers of graph g (its own CSR edge order)."""
    a, b = int(batch.edge_offsets[g]), int(batch.edge_offsets[g + 1])
    return result.truss[a:b]


class CapturedBatch:
    """One batched decomposition recorded as a CUDA graph and replayed.

    Everything a replay touches is allocated at capture: the outputs, the
    workspace (base part plus a fixed triangle-list tail; the device decides
    per replay whether the lists fit) and the per-graph segment ids.  A replay
    re-reads the batch's CSR tensors in place, so new graphs of the same
    shape can be copied into them between replays.  replay() returns the
    per-graph results after checking the run's device status."""

    def __init__(self, batch: GraphBatch, workspace=None, lists="auto", list_budget=None, stream=None):
        from . import _lib
        L = _lib.load()
        g = batch.graph
        rows, cols, rp = T._graph_arrays(g)
        dev = cols.device
        self.batch = batch
        V, E = rp.shape[0] - 1, cols.shape[0]
        self.truss = torch.empty(E, dtype=torch.int32, device=dev)
        self.e_truss = torch.empty(max(E, 1), dtype=torch.int32, device=dev)
        self.cap = E + 2
        self.ptr = torch.empty(self.cap, dtype=torch.int32, device=dev)
        self.stats = torch.zeros(T.STAT_COUNT, dtype=torch.int64, device=dev)
        wso = T._ws_for(dev, workspace)
        base = (L.tdt_decompose_workspace_bytes(V, E) + 255) // 256 * 256
        tail = int(list_budget) if list_budget is not None else T._list_bytes(wso, cols, rp, lists, base, rows)
        self.ws = wso.get(base + tail)
        self.ws_bytes = base + tail
        eo = batch.edge_offsets.to(dev)
        G = batch.num_graphs
        self.seg = torch.repeat_interleave(torch.arange(G, device=dev), eo[1:] - eo[:-1])
        self.kmax = torch.full((G,), 2, dtype=torch.int64, device=dev)
        self.stream = stream or torch.cuda.Stream(dev)
        args = (rows.data_ptr() if rows is not None else None, cols.data_ptr(), rp.data_ptr(), V, E,
                self.truss.data_ptr(), self.e_truss.data_ptr(), self.ptr.data_ptr(), self.cap,
                self.stats.data_ptr(), self.ws.data_ptr(), self.ws_bytes)

        def body():
            s = torch.cuda.current_stream(dev).cuda_stream
            _lib.check(L.tdt_truss_decompose(*args, s), "tdt_truss_decompose")
            self.kmax.fill_(2)
            self.kmax.scatter_reduce_(0, self.seg, self.truss.to(torch.int64), reduce="amax", include_self=True)

        # one eager run on the capture stream (kernel attributes, caches), then capture
        self.stream.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(self.stream):
            body()
        self.stream.synchronize()
        T._check_stats(self.stats.cpu(), "tdt_truss_decompose")
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=self.stream, capture_error_mode="relaxed"):
            body()

    def replay(self, sync=True):
        self.graph.replay()
        if not sync:
            return None
        sh = self.stats.cpu()
        T._check_stats(sh, "tdt_truss_decompose (graph replay)")
        union = T.TrussResult(self.truss, self.e_truss[: int(sh[T.STAT_NETRUSS])], self.ptr[: int(sh[T.STAT_NPTR])],
                              int(sh[T.STAT_KMAX]), int(sh[T.STAT_TRIANGLES]), int(sh[T.STAT_ROUNDS]),
                              bool(sh[T.STAT_LISTED]))
        return BatchResult(self.truss, self.kmax, union)


def capture(batch: GraphBatch, workspace=None, lists="auto", list_budget=None):
    """CUDA-graph capture of decompose(batch) (see CapturedBatch)."""
    return CapturedBatch(batch, workspace=workspace, lists=lists, list_budget=list_budget)
