"""Drop-in replacement of the reference's ``trusstensor`` operator module.

Same 20 operator names, argument orders and in-place semantics as
``PYBIND11_MODULE(trusstensor, m)`` (demo_truss/myops/mysrc/hpu_extension/
myhpu_extension.cpp:572-593), plus the k-truss search operators that the
reference launches from pycuda (ktruss_search/ktruss_cuda.py:316-343).

Every operator takes torch CUDA tensors, returns None and writes its outputs
in place (``segment_isin2*`` accumulate into ``output`` as in the reference).
Work is enqueued on torch's current stream.  Differences from the reference,
all on its failure paths: arguments are checked (dtype int32/bool, CUDA,
contiguous, sizes) and a bad call raises instead of reading out of bounds;
CPU tensors raise (the reference dispatched those to OpenMP twins; this
library has no CPU path).

Operators of the reference's research variants that are outside the
truss-decomposition hot path (undirected/oriented peeling kernels, the
triangle-list and fusion-ablation kernels) are exported and raise
NotImplementedError.
"""
import torch

from . import _lib

__all__ = [
    "segment_add", "segment_isin2", "segment_isin2tile",
    "sub_AllAffectedSupport", "sub_AllAffectedSupport_not", "sub_AllAffectedSupport_notwin",
    "sub_AllAffectedSupport_tile", "sub_AllAffectedSupport_tilenot", "sub_AllAffectedSupport_tilenotwin",
    "segment_isinis_m", "sub_suppport_affect", "peeling_undirect_tile", "peeling_undirect",
    "peeling_direct_oo", "peeling_direct_tile_oo", "peeling_direct_ii", "peeling_direct_tile_ii",
    "peeling_direct_oi", "peeling_direct_tile_oi", "segment_isinmm",
    # k-truss search operators (pycuda entry points in the reference)
    "segment_isin2_k", "segment_isin2tile_k", "sub_AffectedSupport", "sub_AffectedSupport_tile",
]


def _stream():
    return ctypes_stream(torch.cuda.current_stream())


def ctypes_stream(s):
    return s.cuda_stream


def _t(x, name, dtype):
    if not isinstance(x, torch.Tensor):
        raise TypeError("%s must be a torch.Tensor" % name)
    if not x.is_cuda:
        raise TypeError("%s is on %s: tdtdecomposition_gb300 operators run on CUDA tensors only" % (name, x.device))
    if x.dtype != dtype:
        raise TypeError("%s must be %s (got %s)" % (name, dtype, x.dtype))
    if not x.is_contiguous():
        raise ValueError("%s must be contiguous" % name)
    return x.data_ptr()


def _i32(x, name):
    return _t(x, name, torch.int32)


def _u8(x, name):
    return _t(x, name, torch.bool)


def _same_device(*ts):
    d = ts[0].device
    for t in ts[1:]:
        if t.device != d:
            raise ValueError("all tensors must be on the same device (%s vs %s)" % (d, t.device))
    return d


def _call(fn, *args):
    L = _lib.load()
    _lib.check(getattr(L, fn)(*args), fn)


# ------------------------------------------------------------------ hot path
def segment_add(col_indices, col_ptr, output):
    """myhpu_extension.cpp:8-16: output[r] = sum(col_indices[col_ptr[r]:col_ptr[r+1]])
    for the non-empty rows r < len(output)."""
    _same_device(col_indices, col_ptr, output)
    n = output.shape[0]
    if col_ptr.shape[0] < n + 1:
        raise ValueError("col_ptr has %d entries, need %d" % (col_ptr.shape[0], n + 1))
    _call("tdt_segment_add", _i32(col_indices, "col_indices"), col_indices.shape[0], _i32(col_ptr, "col_ptr"),
          _i32(output, "output"), n, _stream())


def segment_isin2(a_rows, b_col_indices, b_row_ptr, output):
    """myhpu_extension.cpp:24-34: output[i] += triangles containing edge i."""
    _same_device(a_rows, b_col_indices, b_row_ptr, output)
    _check_edges(a_rows, b_col_indices, output)
    _call("tdt_segment_isin2", _i32(a_rows, "a_rows"), _i32(b_col_indices, "b_col_indices"),
          _i32(b_row_ptr, "b_row_ptr"), b_row_ptr.shape[0], _i32(output, "output"), output.shape[0], _stream())


def segment_isin2tile(a_rows, b_col_indices, b_row_ptr, n_cut, output):
    """myhpu_extension.cpp:43-56: the tiled support count (same result for any n_cut)."""
    _same_device(a_rows, b_col_indices, b_row_ptr, output)
    _check_edges(a_rows, b_col_indices, output)
    _call("tdt_segment_isin2tile", _i32(a_rows, "a_rows"), _i32(b_col_indices, "b_col_indices"),
          _i32(b_row_ptr, "b_row_ptr"), b_row_ptr.shape[0], int(n_cut), _i32(output, "output"),
          output.shape[0], _stream())


def _check_edges(a_rows, cols, output):
    if a_rows.shape[0] < output.shape[0] or cols.shape[0] < output.shape[0]:
        raise ValueError("output has %d edges but a_rows/b_col_indices hold %d/%d"
                         % (output.shape[0], a_rows.shape[0], cols.shape[0]))


def _affect(fn, e_affect, a_rows, b_col_indices, b_row_ptr, n_cut, mark, l, n_mark, output, win=None):
    _same_device(e_affect, a_rows, b_col_indices, b_row_ptr, mark, n_mark, output)
    E = b_col_indices.shape[0]
    for name, t in (("a_rows", a_rows), ("mark", mark), ("n_mark", n_mark), ("output", output)):
        if t.shape[0] < E:
            raise ValueError("%s has %d entries, fewer than the %d edges" % (name, t.shape[0], E))
    args = [_i32(e_affect, "e_affect"), e_affect.shape[0], _i32(a_rows, "a_rows"),
            _i32(b_col_indices, "b_col_indices"), _i32(b_row_ptr, "b_row_ptr"), b_row_ptr.shape[0]]
    if n_cut is not None:
        args.append(int(n_cut))
    args += [_u8(mark, "mark"), int(l), _u8(n_mark, "n_mark"), _i32(output, "output")]
    if win is not None:
        windows_high, in_windows_mask, buff_index, buf_size = win
        _same_device(output, in_windows_mask, buff_index, buf_size)
        if buff_index.shape[0] < E or in_windows_mask.shape[0] < E or buf_size.shape[0] < 1:
            raise ValueError("window buffers must hold one entry per edge (buf_size: 1)")
        args += [int(windows_high), _u8(in_windows_mask, "in_windows_mask"), _i32(buff_index, "buff_index"),
                 _i32(buf_size, "buf_size")]
    args += [E, _stream()]
    _call(fn, *args)


def sub_AllAffectedSupport(e_affect, a_rows, b_col_indices, b_row_ptr, mark, l, n_mark, output):
    """myhpu_extension.cpp:70-86 (mark = deleted edges)."""
    _affect("tdt_sub_all_affected_support", e_affect, a_rows, b_col_indices, b_row_ptr, None, mark, l, n_mark,
            output)


def sub_AllAffectedSupport_tile(e_affect, a_rows, b_col_indices, b_row_ptr, n_cut, mark, l, n_mark, output):
    """myhpu_extension.cpp:162-177."""
    _affect("tdt_sub_all_affected_support_tile", e_affect, a_rows, b_col_indices, b_row_ptr, n_cut, mark, l,
            n_mark, output)


def sub_AllAffectedSupport_not(e_affect, a_rows, b_col_indices, b_row_ptr, mark, l, n_mark, output):
    """myhpu_extension.cpp:93-106 (mark = alive and not peeled this round)."""
    _affect("tdt_sub_all_affected_support_not", e_affect, a_rows, b_col_indices, b_row_ptr, None, mark, l,
            n_mark, output)


def sub_AllAffectedSupport_tilenot(e_affect, a_rows, b_col_indices, b_row_ptr, n_cut, mark, l, n_mark, output):
    """myhpu_extension.cpp:191-205, the peel update of the `--cuda` flow."""
    _affect("tdt_sub_all_affected_support_tilenot", e_affect, a_rows, b_col_indices, b_row_ptr, n_cut, mark, l,
            n_mark, output)


def sub_AllAffectedSupport_notwin(e_affect, a_rows, b_col_indices, b_row_ptr, mark, l, n_mark, output,
                                  windows_high, in_windows_mask, buff_index, buf_size):
    """myhpu_extension.cpp:123-140."""
    _affect("tdt_sub_all_affected_support_notwin", e_affect, a_rows, b_col_indices, b_row_ptr, None, mark, l,
            n_mark, output, (windows_high, in_windows_mask, buff_index, buf_size))


def sub_AllAffectedSupport_tilenotwin(e_affect, a_rows, b_col_indices, b_row_ptr, n_cut, mark, l, n_mark, output,
                                      windows_high, in_windows_mask, buff_index, buf_size):
    """myhpu_extension.cpp:224-242."""
    _affect("tdt_sub_all_affected_support_tilenotwin", e_affect, a_rows, b_col_indices, b_row_ptr, n_cut, mark, l,
            n_mark, output, (windows_high, in_windows_mask, buff_index, buf_size))


# ------------------------------------------------------------------ k-truss search operators
def segment_isin2_k(a_rows, b_col_indices, b_row_ptr, k, output):
    """ktruss_cuda.py:121-159 (run_kernel_two_k, :316-322)."""
    _same_device(a_rows, b_col_indices, b_row_ptr, output)
    _check_edges(a_rows, b_col_indices, output)
    _call("tdt_segment_isin2_k", _i32(a_rows, "a_rows"), _i32(b_col_indices, "b_col_indices"),
          _i32(b_row_ptr, "b_row_ptr"), b_row_ptr.shape[0], int(k), _i32(output, "output"), output.shape[0],
          _stream())


def segment_isin2tile_k(a_rows, b_col_indices, b_row_ptr, n_cut, k, output):
    """ktruss_cuda.py:160-200 (run_kernel_two_tile_k, :323-329)."""
    _same_device(a_rows, b_col_indices, b_row_ptr, output)
    _check_edges(a_rows, b_col_indices, output)
    _call("tdt_segment_isin2tile_k", _i32(a_rows, "a_rows"), _i32(b_col_indices, "b_col_indices"),
          _i32(b_row_ptr, "b_row_ptr"), b_row_ptr.shape[0], int(n_cut), int(k), _i32(output, "output"),
          output.shape[0], _stream())


def sub_AffectedSupport(sub_rows, sub_columns, sub_row_ptr, mark, sub_support):
    """ktruss_cuda.py:201-242 (run_affect_support, :330-336)."""
    _same_device(sub_rows, sub_columns, sub_row_ptr, mark, sub_support)
    _check_edges(sub_rows, sub_columns, sub_support)
    _call("tdt_sub_affected_support", _i32(sub_rows, "sub_rows"), _i32(sub_columns, "sub_columns"),
          _i32(sub_row_ptr, "sub_row_ptr"), sub_row_ptr.shape[0], _u8(mark, "mark"),
          _i32(sub_support, "sub_support"), sub_support.shape[0], _stream())


def sub_AffectedSupport_tile(sub_rows, sub_columns, sub_row_ptr, n_cut, mark, sub_support):
    """ktruss_cuda.py:243-286 (run_affect_support_tile, :337-343)."""
    _same_device(sub_rows, sub_columns, sub_row_ptr, mark, sub_support)
    _check_edges(sub_rows, sub_columns, sub_support)
    _call("tdt_sub_affected_support_tile", _i32(sub_rows, "sub_rows"), _i32(sub_columns, "sub_columns"),
          _i32(sub_row_ptr, "sub_row_ptr"), sub_row_ptr.shape[0], int(n_cut), _u8(mark, "mark"),
          _i32(sub_support, "sub_support"), sub_support.shape[0], _stream())


# ------------------------------------------------------------------ outside the hot path
def _not_on_path(name, where):
    def op(*args, **kwargs):
        raise NotImplementedError(
            "trusstensor.%s (%s) belongs to the reference's research variants, not to the "
            "truss-decomposition hot path this library replaces" % (name, where))
    op.__name__ = name
    return op


segment_isinis_m = _not_on_path("segment_isinis_m", "kernel.cu:687-737")
sub_suppport_affect = _not_on_path("sub_suppport_affect", "kernel.cu:739-805")
peeling_undirect = _not_on_path("peeling_undirect", "kernel.cu:808-905")
peeling_undirect_tile = _not_on_path("peeling_undirect_tile", "kernel.cu:908-1009")
peeling_direct_oo = _not_on_path("peeling_direct_oo", "kernel.cu:1012-1093")
peeling_direct_tile_oo = _not_on_path("peeling_direct_tile_oo", "kernel.cu:1096-1181")
peeling_direct_ii = _not_on_path("peeling_direct_ii", "kernel.cu:1184-1272")
peeling_direct_tile_ii = _not_on_path("peeling_direct_tile_ii", "kernel.cu:1275-1367")
peeling_direct_oi = _not_on_path("peeling_direct_oi", "kernel.cu:1370-1457")
peeling_direct_tile_oi = _not_on_path("peeling_direct_tile_oi", "kernel.cu:1460-1551")
segment_isinmm = _not_on_path("segment_isinmm", "kernel.cu:1555-1607")
