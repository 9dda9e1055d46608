"""Serving: continuous batching of decomposition and k-truss queries.

A request carries a raw edge list on the host and a query (a full
decomposition, or a k-truss search).  The server

* admits arrived requests in arrival order while their estimated device
  footprint fits the memory budget (150 GB by default);
* ingests admitted requests on a separate stream and thread, all requests
  admitted since the last ingest as one group (one host-to-device copy, one
  grouped device preprocessing); their CSR then stays resident on the device
  until the request completes;
* whenever the device is free, packs EVERY ingested request into one disjoint
  union and decomposes it in one run (batch.decompose) — requests that arrive
  while a batch runs join the next one, so work keeps flowing instead of
  waiting for a full batch;
* answers each request from its slice of the union's truss numbers: the
  decomposition itself, or the k-truss as {e : truss(e) >= k} (exact: the
  k-truss is the set of edges whose truss number is at least k);
* records latency = answer on the host - arrival.

Only one decomposition runs at a time: its peel is a persistent cooperative
kernel that needs every block resident, and two such kernels sharing the GPU
could each wait for the other's blocks.  Overlap comes from ingest (copies and
preprocessing on another stream) and result read-back running beside it.
"""
import queue
import threading
import time

import numpy as np
import torch

from . import batch as B, truss as T
from .graph import CSRCOO
from .preprocess import group_offsets, preprocess_edges


class Request:
    __slots__ = ("id", "arrival", "src", "dst", "query", "graph", "vertices", "answer", "t_done", "bytes",
                 "num_edges", "t_admit", "t_ready")

    def __init__(self, rid, arrival, src, dst, query):
        self.id = rid
        self.arrival = arrival
        self.src = src            # host int32 (pinned)
        self.dst = dst
        self.query = query        # "decompose" or ("ktruss", k)
        self.graph = None
        self.vertices = None
        self.answer = None
        self.t_done = None
        self.t_admit = None
        self.t_ready = None
        self.num_edges = 0
        self.bytes = footprint_bytes(len(src))


def footprint_bytes(num_draws):
    """Upper estimate of a request's device memory while resident: raw edges,
    preprocessing workspace, CSR, and its share of a decomposition workspace
    (the triangle-list tail is a fixed server-wide budget)."""
    return int(num_draws) * (8 + 48 + 16 + 80) + (1 << 20)


def answer_for(query, truss_slice):
    if query == "decompose":
        return truss_slice
    return truss_slice >= int(query[1])


# Workspace tail for triangle lists: the device keeps lists for a batch when
# its 24 T bytes fit, else it runs the search peel (no counting pass first).
DEFAULT_LIST_BUDGET = 24e9


def take_group(inbox, max_draws):
    """The next ingest group: block for one request, then take what is
    already queued while the group holds fewer than max_draws edge draws.
    None in the queue ends the stream.  Returns (group, stop)."""
    group = [inbox.get()]
    draws = len(group[0].src) if group[0] is not None else 0
    while group[-1] is not None and draws < max_draws:
        try:
            r = inbox.get_nowait()
        except queue.Empty:
            break
        group.append(r)
        if r is not None:
            draws += len(r.src)
    stop = group[-1] is None
    return (group[:-1] if stop else group), stop


class TrussServer:
    def __init__(self, device=None, memory_budget=150e9, max_batch_edges=1 << 28, list_budget=DEFAULT_LIST_BUDGET,
                 max_group_draws=1 << 23):
        dev = torch.device(device) if device is not None else torch.device("cuda")
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        self.budget = float(memory_budget)
        self.max_batch_edges = int(max_batch_edges)
        self.max_group_draws = int(max_group_draws)
        self.list_budget = int(list_budget)  # workspace tail for triangle lists (device decides per batch)
        self.ingest_stream = torch.cuda.Stream(self.device)
        self.compute_stream = torch.cuda.Stream(self.device)
        self.ws = T.Workspace(self.device)
        self.pp_ws = T.Workspace(self.device)

    # ------------------------------------------------------------ ingest
    def _ingest_loop(self, inbox, ready):
        """Ingests the requests admitted so far as one group, up to
        max_group_draws edge draws: one host-to-device copy of their
        concatenated edge lists and one grouped preprocessing call (vertex ids
        shifted per request, ranks grouped per request), so a group of small
        requests costs one set of launches.  The cap lets the decomposition of
        a first group start while a burst of arrivals is still being
        ingested."""
        torch.cuda.set_device(self.device)
        with torch.cuda.stream(self.ingest_stream):
            stop = False
            while not stop:
                group, stop = take_group(inbox, self.max_group_draws)
                if group:
                    ready.put(self._ingest_group(group))

    def _ingest_group(self, group):
        nids = []
        for r in group:
            n = int(max(int(r.src.max()), int(r.dst.max()))) + 1 if len(r.src) else 0
            nids.append(n)
        vo = np.concatenate([[0], np.cumsum(nids)]).astype(np.int64)
        if len(group) == 1:
            s_h, d_h = group[0].src, group[0].dst
            vg = None
        else:
            s_h = torch.cat([r.src + int(vo[i]) for i, r in enumerate(group)]).pin_memory()
            d_h = torch.cat([r.dst + int(vo[i]) for i, r in enumerate(group)]).pin_memory()
            vg = torch.from_numpy(np.repeat(np.arange(len(group), dtype=np.int32), nids)).to(self.device)
        s = s_h.to(self.device, non_blocking=True)
        d = d_h.to(self.device, non_blocking=True)
        g, v = preprocess_edges(s, d, vertex_group=vg, num_ids=int(vo[-1]), workspace=self.pp_ws)
        if vg is None:
            veo = (torch.tensor([0, g.num_vertices]), torch.tensor([0, g.num_edges]))
        else:
            a, b = group_offsets(vg, v, g)
            veo = (a.cpu(), b.cpu())
        self.ingest_stream.synchronize()
        t = time.perf_counter()
        for i, r in enumerate(group):
            r.num_edges = int(veo[1][i + 1] - veo[1][i])
            r.t_ready = t
        return (group, B.batch_from_union(g, veo[1], veo[0]))

    # ------------------------------------------------------------ serving loop
    def run(self, requests, real_time=True):
        """Serve `requests` (sorted by arrival, seconds from start).  Returns
        the requests with answers and timing filled in."""
        torch.cuda.set_device(self.device)
        inbox, ready = queue.Queue(), queue.Queue()
        ingest = threading.Thread(target=self._ingest_loop, args=(inbox, ready), daemon=True)
        ingest.start()
        pending = list(requests)
        waiting, resident = [], []
        used = 0.0
        done = 0
        t0 = time.perf_counter()
        self.t0 = t0
        try:
            while done < len(requests):
                now = time.perf_counter() - t0
                while pending and (not real_time or pending[0].arrival <= now):
                    r = pending.pop(0)
                    if not real_time:
                        r.arrival = now  # latency counted from submission
                    waiting.append(r)
                while waiting and used + waiting[0].bytes <= self.budget:
                    r = waiting.pop(0)
                    used += r.bytes
                    r.t_admit = time.perf_counter()
                    inbox.put(r)
                while True:
                    try:
                        resident.append(ready.get_nowait())
                    except queue.Empty:
                        break
                if not resident:
                    if waiting and used == 0.0:
                        raise RuntimeError("request %d does not fit the memory budget" % waiting[0].id)
                    try:
                        resident.append(ready.get(timeout=0.001))
                    except queue.Empty:
                        if real_time and pending and not waiting:
                            time.sleep(max(0.0, min(0.002, pending[0].arrival - (time.perf_counter() - t0))))
                    continue
                # one batch: every ingested chunk (up to max_batch_edges)
                chunks, edges = [], 0
                for ch in resident:
                    e = ch[1].graph.num_edges
                    if chunks and edges + e > self.max_batch_edges:
                        break
                    chunks.append(ch)
                    edges += e
                resident = resident[len(chunks):]
                self._run_batch(chunks)
                for reqs, _ in chunks:
                    for r in reqs:
                        used -= r.bytes
                    done += len(reqs)
        finally:
            inbox.put(None)
            ingest.join(timeout=30)
        return requests

    def _run_batch(self, chunks):
        with torch.cuda.stream(self.compute_stream):
            for _, bt in chunks:  # made on the ingest stream, read on this one
                for t in (bt.graph.columns, bt.graph.rows, bt.graph.row_ptr):
                    t.record_stream(self.compute_stream)
            if len(chunks) == 1:
                bt = chunks[0][1]
            else:
                bt = pack_device([c[1].graph for c in chunks], self.device)
            res = B.decompose(bt, workspace=self.ws, list_budget=self.list_budget)
            # per-request edge ranges inside the packed union
            batch, eo = [], [0]
            ebase = bt.edge_offsets.tolist()
            for ci, (reqs, cb) in enumerate(chunks):
                ceo = cb.edge_offsets.tolist()
                for i, r in enumerate(reqs):
                    batch.append(r)
                    eo.append(ebase[ci] + ceo[i + 1])
            outs = []
            for i, r in enumerate(batch):
                a = answer_for(r.query, res.truss[eo[i]:eo[i + 1]])
                h = torch.empty(a.shape, dtype=a.dtype, pin_memory=True)
                h.copy_(a, non_blocking=True)
                outs.append(h)
            self.compute_stream.synchronize()
            t = time.perf_counter() - self.t0
            for r, h in zip(batch, outs):
                r.answer = h
                r.t_done = t


def pack_device(graphs, device):
    """Disjoint union of device CSRCOOs (int64 row offsets)."""
    nv = [g.num_vertices for g in graphs]
    ne = [g.num_edges for g in graphs]
    vo = np.concatenate([[0], np.cumsum(nv)]).astype(np.int64)
    eo = np.concatenate([[0], np.cumsum(ne)]).astype(np.int64)
    cols = torch.cat([g.columns + int(vo[i]) for i, g in enumerate(graphs)]) if graphs else torch.zeros(0, dtype=torch.int32, device=device)
    rows = torch.cat([g.rows + int(vo[i]) for i, g in enumerate(graphs)]) if graphs else torch.zeros(0, dtype=torch.int32, device=device)
    rp = torch.cat([g.row_ptr[:-1].to(torch.int64) + int(eo[i]) for i, g in enumerate(graphs)] +
                   [torch.tensor([eo[-1]], dtype=torch.int64, device=device)])
    return B.GraphBatch(CSRCOO(columns=cols.to(torch.int32), row_ptr=rp, rows=rows.to(torch.int32)),
                        torch.from_numpy(vo), torch.from_numpy(eo))


def make_requests(specs, device=None):
    """Host edge lists (pinned) for request specs from workloads.request_stream."""
    from . import generators as G
    reqs = []
    for sp in specs:
        gen = sp["gen"]
        if gen["kind"] == "ba":
            s, d = G.ba_edges(gen["n"], gen["m"], gen["seed"])
            s, d = torch.from_numpy(s), torch.from_numpy(d)
        else:
            s, d = G.rmat_edges_device(gen["scale"], 16 << gen["scale"], seed=gen["seed"], device=device or "cuda")
            s, d = s.cpu(), d.cpu()
        reqs.append(Request(sp["id"], sp["arrival"], s.pin_memory(), d.pin_memory(), sp["query"]))
    return reqs


def latency_stats(requests):
    lat = np.array([r.t_done - r.arrival for r in requests])
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3)}
