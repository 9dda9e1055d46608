"""Graph preprocessing: edge list -> degree-oriented CSRCOO.

Restates read_prepro_save (singlegpu_truss.py:172-178) = Graph.read_edgelist
(src/type/Graph_Truss.py:177-213) + CSRCOO.edge_list_to_Graph
(src/type/CSRCOO.py:128-162): drop self-loops, dedup unordered pairs, rank
vertices by (degree, id) — the reference ranks by degree with numpy's
unstable argsort, so ties are broken by id here (the results that matter,
truss numbers keyed by original vertex pair, do not depend on the tie
order) — relabel by rank, orient low->high, CSR sorted by (row, column).

All steps run on the GPU (edge lists already in device memory).
"""
import torch

from .graph import CSRCOO


def preprocess_edges(src, dst):
    """src, dst: int32 CUDA tensors of the raw edge list.  Returns
    (CSRCOO with int64 row_ptr, vertices: int32 original id of each rank)."""
    if not src.is_cuda:
        raise TypeError("preprocess_edges runs on CUDA tensors")
    s = src.to(torch.int64)
    d = dst.to(torch.int64)
    keep = s != d
    s, d = s[keep], d[keep]
    lo = torch.minimum(s, d)
    hi = torch.maximum(s, d)
    key = torch.unique(lo * (1 << 32) + hi)             # dedup unordered pairs (sorted)
    lo = key >> 32
    hi = key & 0xFFFFFFFF
    ends = torch.cat([lo, hi])
    ids, deg = torch.unique(ends, return_counts=True)   # vertices present, ascending id
    order = torch.argsort(deg * (1 << 32) + ids)        # rank by (degree, id)
    vertices = ids[order]
    rank = torch.empty_like(order)
    rank[order] = torch.arange(order.numel(), device=order.device)
    ru = rank[torch.searchsorted(ids, lo)]
    rv = rank[torch.searchsorted(ids, hi)]
    a = torch.minimum(ru, rv)
    b = torch.maximum(ru, rv)
    key2, _ = torch.sort(a * (1 << 32) + b)
    rows = (key2 >> 32).to(torch.int32)
    cols = (key2 & 0xFFFFFFFF).to(torch.int32)
    V = vertices.numel()
    rp = torch.zeros(V + 1, dtype=torch.int64, device=src.device)
    rp[1:] = torch.cumsum(torch.bincount(rows.to(torch.int64), minlength=V), 0)
    return CSRCOO(columns=cols, row_ptr=rp, rows=rows), vertices.to(torch.int32)


def wedge_work(graph):
    """W = sum over edges (u,v) of d+(u) + d+(v): the merge work of the
    support pass, used for the algorithmic-bytes roofline
    (B_sup = 4 W + 28 E + 4 (V+1))."""
    rp = graph.row_ptr.to(torch.int64)
    dplus = rp[1:] - rp[:-1]
    return int((dplus[graph.rows.long()] + dplus[graph.columns.long()]).sum())
