"""The oriented graph container, mirroring the reference's ``CSRCOO``
(src/type/CSRCOO.py:9-116): ``columns`` (heads, sorted within a row),
``rows`` (tails, the COO row of each edge) and ``row_ptr`` (CSR offsets of the
rows, or the tiled offsets built by :func:`tiling_row_ptr`).
"""
import torch


class CSRCOO:
    """Degree-oriented CSR + COO rows (every edge stored once, rows[i] < columns[i])."""

    def __init__(self, columns=None, row_ptr=None, rows=None):
        self.columns = columns
        self.row_ptr = row_ptr
        self.rows = rows

    @property
    def num_vertices(self):
        """number of vertices (CSRCOO.py:35-41: row_ptr length - 1)."""
        return self.row_ptr.shape[0] - 1 if hasattr(self.row_ptr, "shape") else 0

    @property
    def num_edges(self):
        return self.columns.shape[0] if hasattr(self.columns, "shape") else 0

    @property
    def device(self):
        if self.columns.device != self.row_ptr.device:
            raise AssertionError("Graph is not on the same device.")
        return self.columns.device

    def to(self, *args, **kwargs):
        self.columns = self.columns.to(*args, **kwargs)
        self.row_ptr = self.row_ptr.to(*args, **kwargs)
        self.rows = self.rows.to(*args, **kwargs)
        return self

    def pin_memory(self):
        self.columns = self.columns.pin_memory()
        self.row_ptr = self.row_ptr.pin_memory()
        self.rows = self.rows.pin_memory()
        return self

    @staticmethod
    def from_numpy(rows, columns, row_ptr, device="cpu"):
        return CSRCOO(columns=torch.as_tensor(columns, dtype=torch.int32, device=device),
                      row_ptr=torch.as_tensor(row_ptr, device=device),
                      rows=torch.as_tensor(rows, dtype=torch.int32, device=device))


def tiling_row_ptr(graph, n_cut):
    """Tiled row offsets (csr_to_tilingcsr, singlegpu_truss.py:160-169): tile
    j of vertex u holds the out-neighbours w with w // (V // n_cut + 1) == j;
    returns int32[V*n_cut + 1].  Computed with torch ops on the graph's device."""
    V = graph.num_vertices
    cols = graph.columns.to(torch.int64)
    rows = graph.rows.to(torch.int64)
    if n_cut == 1:
        block = rows
    else:
        block = cols // (V // n_cut + 1) + rows * n_cut
    cnt = torch.bincount(block, minlength=V * n_cut)
    out = torch.zeros(V * n_cut + 1, dtype=torch.int32, device=graph.columns.device)
    out[1:] = torch.cumsum(cnt, 0).to(torch.int32)
    return out
