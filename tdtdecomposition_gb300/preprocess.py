"""Graph preprocessing: edge list -> degree-oriented CSRCOO.

Restates read_prepro_save (singlegpu_truss.py:172-178) = Graph.read_edgelist
(src/type/Graph_Truss.py:177-213) + CSRCOO.edge_list_to_Graph
(src/type/CSRCOO.py:128-162): drop self-loops, dedup unordered pairs, rank
vertices by (degree, id) — the reference ranks by degree with numpy's
unstable argsort, so ties are broken by id here (the results that matter,
truss numbers keyed by original vertex pair, do not depend on the tie
order) — relabel by rank, orient low->high, CSR sorted by (row, column).

All steps run on the GPU (edge lists already in device memory): the kernels
are in csrc/preprocess.cu (tdt_preprocess).
"""
import torch

from . import _lib
from .graph import CSRCOO


def preprocess_edges(src, dst, vertex_group=None, num_ids=None, workspace=None):
    """src, dst: int32 CUDA tensors of the raw edge list (ids >= 0).  Returns
    (CSRCOO with int64 row_ptr, vertices: int32 original id of each rank),
    computed by tdt_preprocess (own radix sorts and scans, no host sync
    inside; one sync at the end to read the output sizes).

    vertex_group (optional, int32 CUDA tensor indexed by vertex id): a batch
    of graphs with disjoint vertex ids; vertices are then ranked by
    (group, degree, id), so every graph keeps a contiguous range of ranks and
    of CSR rows/edges in group order."""
    if not (src.is_cuda and dst.is_cuda):
        raise TypeError("preprocess_edges runs on CUDA tensors")
    L = _lib.load()
    src = src.to(torch.int32).contiguous()
    dst = dst.to(torch.int32).contiguous()
    dev = src.device
    m = src.numel()
    if num_ids is None:
        num_ids = int(torch.maximum(src.max(), dst.max())) + 1 if m else 0
    ng = 0
    if vertex_group is not None:
        vertex_group = vertex_group.to(torch.int32).contiguous()
        ng = int(vertex_group.max()) + 1 if vertex_group.numel() else 1
        if vertex_group.numel() < num_ids:
            raise ValueError("vertex_group must hold one entry per vertex id")
    rows = torch.empty(max(m, 1), dtype=torch.int32, device=dev)
    cols = torch.empty(max(m, 1), dtype=torch.int32, device=dev)
    rp = torch.empty(num_ids + 1, dtype=torch.int64, device=dev)
    verts = torch.empty(max(num_ids, 1), dtype=torch.int32, device=dev)
    counts = torch.zeros(3, dtype=torch.int64, device=dev)
    need = L.tdt_preprocess_workspace_bytes(m, num_ids)
    ws = (workspace.get(need) if workspace is not None
          else torch.empty(need, dtype=torch.uint8, device=dev))
    with torch.cuda.device(dev):
        rc = L.tdt_preprocess(src.data_ptr(), dst.data_ptr(), m, num_ids,
                              vertex_group.data_ptr() if vertex_group is not None else None, ng,
                              rows.data_ptr(), cols.data_ptr(), rp.data_ptr(), verts.data_ptr(), counts.data_ptr(),
                              ws.data_ptr(), ws.numel(), torch.cuda.current_stream(dev).cuda_stream)
    _lib.check(rc, "tdt_preprocess")
    E, V, st = (int(x) for x in counts.cpu())
    if st != 0:
        raise _lib.TdtError(st, "tdt_preprocess", "vertex id outside [0, num_ids)")
    g = CSRCOO(columns=cols[:E], row_ptr=rp[:V + 1].clone(), rows=rows[:E])
    return g, verts[:V]


def group_offsets(vertex_group, vertices, graph):
    """For a batch preprocessed with vertex_group: (vertex_offsets,
    edge_offsets) int64[G+1] of each graph's contiguous rank and edge ranges
    (graphs without edges get empty ranges)."""
    G = int(vertex_group.max()) + 1 if vertex_group.numel() else 0
    cnt = torch.bincount(vertex_group.to(torch.int64)[vertices.long()], minlength=G)
    vo = torch.zeros(G + 1, dtype=torch.int64, device=cnt.device)
    vo[1:] = torch.cumsum(cnt, 0)
    eo = graph.row_ptr.to(torch.int64)[vo]
    return vo, eo


def wedge_work(graph):
    """W = sum over edges (u,v) of d+(u) + d+(v): the merge work of the
    support pass, used for the algorithmic-bytes roofline
    (B_sup = 4 W + 28 E + 4 (V+1))."""
    rp = graph.row_ptr.to(torch.int64)
    dplus = rp[1:] - rp[:-1]
    return int((dplus[graph.rows.long()] + dplus[graph.columns.long()]).sum())
