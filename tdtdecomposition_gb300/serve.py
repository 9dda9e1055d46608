"""Serving: continuous batching of decomposition and k-truss queries.

A request carries a raw edge list on the host and a query (a full
decomposition, a k-truss search, or -- on a resident graph -- a triangle
count), or names a graph already resident on the server (a handle).  The
server

* admits arrived requests in arrival order while their estimated device
  footprint fits the memory budget (150 GB by default);
* ingests admitted requests on a separate stream and thread, all requests
  admitted since the last ingest as one group (one host-to-device copy, one
  grouped device preprocessing); their CSR then stays resident on the device
  until the request completes;
* whenever the device is free, picks the next work: queries on resident
  graphs first (answered from their cached truss numbers, or by one call on
  the resident CSR); then a k-truss query on a large graph alone, by the
  fixed-level peel of ktruss_search (ktruss_search/ktruss_cuda.py:383-463),
  which touches only the low-support edges instead of decomposing the whole
  graph; otherwise one disjoint union of the ingested requests, smallest
  first (requests that have waited past max_wait_s go first), up to
  max_batch_edges edges, decomposed in one run (batch.decompose) -- so small
  requests do not wait behind a large graph's peel, and requests that arrive
  while a batch runs join a later one;
* answers each request from its slice of the union's truss numbers: the
  decomposition itself, or the k-truss as {e : truss(e) >= k} (exact: the
  k-truss is the set of edges whose truss number is at least k);
* keeps the graph of a request submitted with keep=True resident under its
  handle (its CSR and truss numbers, least recently used evicted first past
  resident_budget), so later queries on it need no ingest and, once decomposed,
  no kernel at all;
* records latency = answer on the host - arrival, and how each request was
  answered (``path``: "batch", "search" or "resident").

Only one peel runs at a time: it is a persistent cooperative kernel that needs
every block resident, and two such kernels sharing the GPU could each wait for
the other's blocks.  Overlap comes from ingest (copies and preprocessing on
another stream) and result read-back running beside it.
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
                 "num_edges", "t_admit", "t_ready", "handle", "keep", "path")

    def __init__(self, rid, arrival, src, dst, query, handle=None, keep=False):
        self.id = rid
        self.arrival = arrival
        self.src = src            # host int32 (pinned); None for a query on a resident graph
        self.dst = dst
        self.query = query        # "decompose", ("ktruss", k) or, on a resident graph, "triangles"
        self.handle = handle      # resident graph to query (src is None) or to keep this graph under
        self.keep = bool(keep)
        self.path = None          # how it was answered: "batch", "search" or "resident"
        self.graph = None
        self.vertices = None
        self.answer = None
        self.t_done = None
        self.t_admit = None
        self.t_ready = None
        self.num_edges = 0
        self.bytes = footprint_bytes(len(src)) if src is not None else 0


def footprint_bytes(num_draws):
    """Upper estimate of a request's device memory while resident: raw edges,
    preprocessing workspace, CSR, and its share of a decomposition workspace
    (the triangle-list tail is a fixed server-wide budget)."""
    return int(num_draws) * (8 + 48 + 16 + 80) + (1 << 20)


def answer_for(query, truss_slice):
    if query == "decompose":
        return truss_slice
    return truss_slice >= int(query[1])


def is_ktruss(query):
    return isinstance(query, tuple) and query[0] == "ktruss"


class Resident:
    """A graph kept on the device between queries: its CSR and, once known,
    its truss numbers."""
    __slots__ = ("graph", "truss", "bytes")

    def __init__(self, graph, truss=None):
        self.graph = graph
        self.truss = truss
        self.bytes = 16 * graph.num_edges + 8 * (graph.num_vertices + 1)


# Workspace tail for triangle lists: the device keeps lists for a batch when
# its 24 T bytes fit, else it runs the search peel (no counting pass first).
DEFAULT_LIST_BUDGET = 24e9


def take_group(inbox, max_draws, alone=None, carry=None):
    """The next ingest group: block for one request, then take what is
    already queued while the group holds fewer than max_draws edge draws.
    None in the queue ends the stream.  A request for which alone(r) holds
    forms a group of its own: met inside a group, it is kept in `carry` (a
    list) and starts the next one.  Returns (group, stop)."""
    group = [carry.pop(0) if carry else inbox.get()]
    if group[0] is not None and alone is not None and alone(group[0]):
        return group, False
    draws = len(group[0].src) if group[0] is not None else 0
    while group[-1] is not None and draws < max_draws:
        try:
            r = inbox.get_nowait()
        except queue.Empty:
            break
        if r is not None and alone is not None and alone(r):
            carry.append(r)
            break
        group.append(r)
        if r is not None:
            draws += len(r.src)
    stop = group[-1] is None
    return (group[:-1] if stop else group), stop


class TrussServer:
    """Continuous-batching server on one GPU.

    memory_budget: device bytes the admitted requests may hold (estimated by
    footprint_bytes); max_batch_edges: edges of one union (bounds the time a
    union's peel holds the device, so the latency of the requests behind it);
    max_wait_s: a request waiting longer goes into the next union first;
    search_min_edges: k-truss queries on graphs with at least this many edges
    run the fixed-level search alone; resident_budget: device bytes of the
    graphs kept under handles (least recently used evicted first)."""

    def __init__(self, device=None, memory_budget=150e9, max_batch_edges=1 << 23, list_budget=DEFAULT_LIST_BUDGET,
                 max_group_draws=1 << 23, max_wait_s=0.25, search_min_edges=1 << 19, resident_budget=20e9):
        dev = torch.device(device) if device is not None else torch.device("cuda")
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        self.budget = float(memory_budget)
        self.max_batch_edges = int(max_batch_edges)
        self.max_group_draws = int(max_group_draws)
        self.max_wait_s = float(max_wait_s)
        self.search_min_edges = int(search_min_edges)
        self.resident_budget = float(resident_budget)
        self.list_budget = int(list_budget)  # workspace tail for triangle lists (device decides per batch)
        self.ingest_stream = torch.cuda.Stream(self.device)
        self.compute_stream = torch.cuda.Stream(self.device)
        self.ws = T.Workspace(self.device)
        self.pp_ws = T.Workspace(self.device)
        self.resident = {}          # handle -> Resident, in least-recently-used order
        self.resident_bytes = 0

    # ------------------------------------------------------------ ingest
    def _ingest_loop(self, inbox, ready):
        """Ingests the requests admitted so far as one group, up to
        max_group_draws edge draws: one host-to-device copy of their
        concatenated edge lists and one grouped preprocessing call (vertex ids
        shifted per request, ranks grouped per request), so a group of small
        requests costs one set of launches.  The cap lets the decomposition of
        a first group start while a burst of arrivals is still being
        ingested.  Large k-truss queries are ingested alone (the search
        path)."""
        torch.cuda.set_device(self.device)
        carry = []
        with torch.cuda.stream(self.ingest_stream):
            stop = False
            while not stop:
                group, stop = take_group(inbox, self.max_group_draws, self._search_candidate, carry)
                if group:
                    ready.put(self._ingest_group(group))

    def _search_candidate(self, r):
        """A k-truss query whose edge list may reach search_min_edges edges
        after preprocessing: ingested alone, so it can take the search path."""
        return is_ktruss(r.query) and len(r.src) >= self.search_min_edges

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
        waiting, resident_q, chunks = [], [], []
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
                    (resident_q if r.src is None else waiting).append(r)
                while waiting and used + waiting[0].bytes <= self.budget:
                    r = waiting.pop(0)
                    used += r.bytes
                    r.t_admit = time.perf_counter()
                    inbox.put(r)
                while True:
                    try:
                        chunks.append(ready.get_nowait())
                    except queue.Empty:
                        break
                if resident_q:
                    for r in resident_q:
                        self._serve_resident(r)
                    done += len(resident_q)
                    resident_q = []
                    continue
                if not chunks:
                    if waiting and used == 0.0:
                        raise RuntimeError("request %d does not fit the memory budget" % waiting[0].id)
                    try:
                        chunks.append(ready.get(timeout=0.001))
                    except queue.Empty:
                        if real_time and pending and not waiting:
                            time.sleep(max(0.0, min(0.002, pending[0].arrival - (time.perf_counter() - t0))))
                    continue
                work, chunks = self._pick(chunks, time.perf_counter() - t0)
                if len(work) == 1 and len(work[0][0]) == 1 and self._searches(work[0][0][0]):
                    self._run_search(work[0])
                else:
                    self._run_batch(work)
                for reqs, _ in work:
                    for r in reqs:
                        used -= r.bytes
                    done += len(reqs)
        finally:
            inbox.put(None)
            ingest.join(timeout=30)
        return requests

    def _searches(self, r):
        return is_ktruss(r.query) and r.num_edges >= self.search_min_edges

    def _pick(self, chunks, now):
        """The next work among the ingested chunks: a lone large k-truss query
        (fixed-level search), else a union of chunks up to max_batch_edges
        edges, those holding a request older than max_wait_s first, then the
        smallest.  Returns (work, remaining chunks)."""
        for i, ch in enumerate(chunks):
            if len(ch[0]) == 1 and self._searches(ch[0][0]):
                return [ch], chunks[:i] + chunks[i + 1:]

        def key(ch):
            oldest = min(r.arrival for r in ch[0])
            return (0 if now - oldest > self.max_wait_s else 1, ch[1].graph.num_edges, oldest)

        order = sorted(range(len(chunks)), key=lambda i: key(chunks[i]))
        take, edges = [], 0
        for i in order:
            e = chunks[i][1].graph.num_edges
            if take and edges + e > self.max_batch_edges:
                continue
            take.append(i)
            edges += e
        taken = set(take)
        return [chunks[i] for i in sorted(take)], [c for i, c in enumerate(chunks) if i not in taken]

    def _finish(self, reqs, outs, path):
        self.compute_stream.synchronize()
        t = time.perf_counter() - self.t0
        for r, h in zip(reqs, outs):
            r.answer = h
            r.t_done = t
            r.path = path

    @staticmethod
    def _to_host(a):
        h = torch.empty(a.shape, dtype=a.dtype, pin_memory=True)
        h.copy_(a, non_blocking=True)
        return h

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
            # per-request vertex and edge ranges inside the packed union
            batch, vr, er = [], [], []
            ebase, vbase = bt.edge_offsets.tolist(), bt.vertex_offsets.tolist()
            for ci, (reqs, cb) in enumerate(chunks):
                ceo, cvo = cb.edge_offsets.tolist(), cb.vertex_offsets.tolist()
                for i, r in enumerate(reqs):
                    batch.append(r)
                    er.append((ebase[ci] + ceo[i], ebase[ci] + ceo[i + 1]))
                    vr.append((vbase[ci] + cvo[i], vbase[ci] + cvo[i + 1]))
            outs = []
            for r, (a, b), (va, vb) in zip(batch, er, vr):
                tr = res.truss[a:b]
                outs.append(self._to_host(answer_for(r.query, tr)))
                if r.keep:
                    g = bt.graph
                    sub = CSRCOO(columns=g.columns[a:b] - int(va), row_ptr=g.row_ptr[va:vb + 1] - int(a),
                                 rows=g.rows[a:b] - int(va))
                    self._keep(r.handle, sub, tr.clone())
            self._finish(batch, outs, "batch")

    def _run_search(self, chunk):
        """One large k-truss query alone: the fixed-level peel on its graph."""
        (r,), bt = chunk
        with torch.cuda.stream(self.compute_stream):
            for t in (bt.graph.columns, bt.graph.rows, bt.graph.row_ptr):
                t.record_stream(self.compute_stream)
            mask = T.ktruss_search(bt.graph, int(r.query[1]), workspace=self.ws, stream=self.compute_stream,
                                   lists=False)
            if r.keep:
                self._keep(r.handle, bt.graph, None)
            self._finish([r], [self._to_host(mask)], "search")

    # ------------------------------------------------------------ resident graphs
    def _keep(self, handle, graph, truss):
        if handle is None:
            raise ValueError("keep=True needs a handle")
        old = self.resident.pop(handle, None)
        if old is not None:
            self.resident_bytes -= old.bytes
        rs = Resident(graph, truss)
        self.resident[handle] = rs
        self.resident_bytes += rs.bytes
        while self.resident_bytes > self.resident_budget and len(self.resident) > 1:
            h = next(iter(self.resident))
            self.resident_bytes -= self.resident.pop(h).bytes

    def _serve_resident(self, r):
        """A query on a resident graph: from its cached truss numbers when the
        graph was decomposed, else one call on its resident CSR (the
        decomposition's truss numbers are cached for the next query)."""
        rs = self.resident.pop(r.handle, None)
        if rs is None:
            raise KeyError("graph %r is not resident on the server" % (r.handle,))
        self.resident[r.handle] = rs  # most recently used
        r.num_edges = rs.graph.num_edges
        with torch.cuda.stream(self.compute_stream):
            if r.query == "triangles":
                a = torch.tensor([T.triangle_count(rs.graph, workspace=self.ws, stream=self.compute_stream)])
            elif rs.truss is None and is_ktruss(r.query):
                a = T.ktruss_search(rs.graph, int(r.query[1]), workspace=self.ws, stream=self.compute_stream,
                                    lists=False)
            else:
                if rs.truss is None:
                    rs.truss = T.truss_decompose(rs.graph, workspace=self.ws, stream=self.compute_stream,
                                                 list_budget=self.list_budget).truss
                a = answer_for(r.query, rs.truss)
            self._finish([r], [self._to_host(a)], "resident")

    def register(self, handle, graph):
        """Keep an already preprocessed device graph resident under `handle`."""
        self._keep(handle, graph, None)


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


SIZE_CLASSES = (("small (E < 2^16)", 0, 1 << 16), ("medium (2^16 <= E < 2^20)", 1 << 16, 1 << 20),
                ("large (E >= 2^20)", 1 << 20, 1 << 62))


def latency_by_class(requests):
    """latency_stats per request-size class (edges after preprocessing)."""
    out = {}
    for name, lo, hi in SIZE_CLASSES:
        rs = [r for r in requests if lo <= r.num_edges < hi]
        if rs:
            out[name] = dict(latency_stats(rs), requests=len(rs))
    return out
