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

The research-variant operators (segment_isinis_m, sub_suppport_affect,
segment_isinmm and the undirected/oriented peel updates) are implemented too;
their drivers are restated in ``flow.py``.
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
    # the operators launch on the current device and its current stream, as
    # the reference's do; tensors of another device would be handed to it
    if d.type == "cuda" and d.index is not None and d.index != torch.cuda.current_device():
        raise ValueError("tensors are on %s but the current device is cuda:%d (use torch.cuda.device)"
                         % (d, torch.cuda.current_device()))
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


# ------------------------------------------------------------------ research-variant operators
def _rows_mask(fn, a_cols, a_ptr, b_cols, b_ptr, m1, m2):
    _same_device(a_cols, a_ptr, b_cols, b_ptr, m1, m2)
    n = max(a_ptr.shape[0] - 1, 0)
    if b_ptr.shape[0] < n + 1:
        raise ValueError("the second row-pointer array has %d entries, need %d" % (b_ptr.shape[0], n + 1))
    if m1.shape[0] < a_cols.shape[0] or m2.shape[0] < b_cols.shape[0]:
        raise ValueError("each mask needs one entry per value of its columns")
    _call(fn, _i32(a_cols, "a_columns"), a_cols.shape[0], _i32(a_ptr, "a_row_ptr"), _i32(b_cols, "b_columns"),
          b_cols.shape[0], _i32(b_ptr, "b_row_ptr"), n, _u8(m1, "mask1"), _u8(m2, "mask2"), _stream())


def segment_isinis_m(a_columns, a_row_ptr, b_columns, b_row_ptr, mask1, mask2):
    """myhpu_extension.cpp:255-265 (kernel.cu:687-737): per row r, set mask1/mask2
    at the positions of the values rows r of a and b share (-1 excepted)."""
    _rows_mask("tdt_segment_isinis_m", a_columns, a_row_ptr, b_columns, b_row_ptr, mask1, mask2)


def segment_isinmm(u_clos, v_clos, uptr, vptr, u_mask, v_mask):
    """myhpu_extension.cpp:555-565 (kernel.cu:1555-1607): segment_isinis_m
    without the -1 exception."""
    _same_device(u_clos, v_clos, uptr, vptr, u_mask, v_mask)
    n = max(uptr.shape[0] - 1, 0)
    if vptr.shape[0] < n + 1:
        raise ValueError("vptr has %d entries, need %d" % (vptr.shape[0], n + 1))
    if u_mask.shape[0] < u_clos.shape[0] or v_mask.shape[0] < v_clos.shape[0]:
        raise ValueError("each mask needs one entry per value of its columns")
    _call("tdt_segment_isinmm", _i32(u_clos, "u_clos"), u_clos.shape[0], _i32(v_clos, "v_clos"), v_clos.shape[0],
          _i32(uptr, "uptr"), _i32(vptr, "vptr"), n, _u8(u_mask, "u_mask"), _u8(v_mask, "v_mask"), _stream())


def sub_suppport_affect(left_nbr, right_nbr, e_curr_rep, support, mask1, mask2, e_affect_mask, l):
    """myhpu_extension.cpp:284-296 (kernel.cu:739-805): per triangle i of
    e_curr_rep[i], decrement the flagged partner edges (one flagged: only when
    e_curr_rep[i] is below the other partner) and flag them in e_affect_mask."""
    _same_device(left_nbr, right_nbr, e_curr_rep, support, mask1, mask2, e_affect_mask)
    n = left_nbr.shape[0]
    for name, t in (("right_nbr", right_nbr), ("e_curr_rep", e_curr_rep), ("mask1", mask1), ("mask2", mask2)):
        if t.shape[0] < n:
            raise ValueError("%s has %d entries, fewer than left_nbr's %d" % (name, t.shape[0], n))
    if e_affect_mask.shape[0] < support.shape[0]:
        raise ValueError("e_affect_mask needs one entry per edge")
    _call("tdt_sub_suppport_affect", _i32(left_nbr, "left_nbr"), _i32(right_nbr, "right_nbr"),
          _i32(e_curr_rep, "e_curr_rep"), n, _i32(support, "support"), support.shape[0], _u8(mask1, "mask1"),
          _u8(mask2, "mask2"), _u8(e_affect_mask, "e_affect_mask"), int(l), _stream())


def _peel_common(e_curr, rows, columns, support, e_mask, n_mark, in_curr, extra):
    _same_device(e_curr, rows, columns, support, e_mask, n_mark, in_curr, *extra)
    E = columns.shape[0]
    for name, t in (("rows", rows), ("support", support), ("e_mask", e_mask), ("n_mark", n_mark),
                    ("in_curr", in_curr)):
        if t.shape[0] < E:
            raise ValueError("%s has %d entries, fewer than the %d edges" % (name, t.shape[0], E))
    return E, [_i32(e_curr, "e_curr"), e_curr.shape[0], _i32(rows, "rows"), _i32(columns, "columns")]


def _tail(support, e_mask, n_mark, in_curr):
    return [_i32(support, "support"), _u8(e_mask, "e_mask"), _u8(n_mark, "n_mark"), _u8(in_curr, "in_curr")]


def _undirect(fn, e_curr, rows, columns, columns_g, row_ptr, edges_id_nbr, support, e_mask, n_mark, in_curr, l,
              n_cut):
    E, args = _peel_common(e_curr, rows, columns, support, e_mask, n_mark, in_curr,
                           (columns_g, row_ptr, edges_id_nbr))
    if edges_id_nbr.shape[0] < columns_g.shape[0]:
        raise ValueError("edges_id_nbr needs one entry per value of columns_g")
    args += [_i32(columns_g, "columns_g"), _i32(row_ptr, "row_ptr"), row_ptr.shape[0],
             _i32(edges_id_nbr, "edges_id_nbr"), columns_g.shape[0]] + _tail(support, e_mask, n_mark, in_curr)
    args += [int(l)] + ([] if n_cut is None else [int(n_cut)]) + [E, _stream()]
    _call(fn, *args)


def peeling_undirect(e_curr, rows, columns, columns_g, row_ptr, edges_id_nbr, support, e_mask, n_mark, in_curr, l):
    """myhpu_extension.cpp:316-331 (kernel.cu:808-905): peel update over the
    symmetric adjacency (columns_g, edges_id_nbr, row_ptr)."""
    _undirect("tdt_peeling_undirect", e_curr, rows, columns, columns_g, row_ptr, edges_id_nbr, support, e_mask,
              n_mark, in_curr, l, None)


def peeling_undirect_tile(e_curr, rows, columns, columns_g, row_ptr, edges_id_nbr, support, e_mask, n_mark, in_curr,
                          l, n_cut):
    """myhpu_extension.cpp:348-363 (kernel.cu:908-1009): the tiled form."""
    _undirect("tdt_peeling_undirect_tile", e_curr, rows, columns, columns_g, row_ptr, edges_id_nbr, support, e_mask,
              n_mark, in_curr, l, n_cut)


def _oo(fn, e_curr, rows, columns, row_ptr, support, e_mask, n_mark, in_curr, l, n_cut):
    E, args = _peel_common(e_curr, rows, columns, support, e_mask, n_mark, in_curr, (row_ptr,))
    args += [_i32(row_ptr, "row_ptr"), row_ptr.shape[0]] + _tail(support, e_mask, n_mark, in_curr)
    args += [int(l)] + ([] if n_cut is None else [int(n_cut)]) + [E, _stream()]
    _call(fn, *args)


def peeling_direct_oo(e_curr, rows, columns, row_ptr, support, e_mask, n_mark, in_curr, l):
    """myhpu_extension.cpp:377-390 (kernel.cu:1012-1093): third vertex in the
    out-lists of both ends."""
    _oo("tdt_peeling_direct_oo", e_curr, rows, columns, row_ptr, support, e_mask, n_mark, in_curr, l, None)


def peeling_direct_tile_oo(e_curr, rows, columns, row_ptr, support, e_mask, n_mark, in_curr, l, n_cut):
    """myhpu_extension.cpp:405-418 (kernel.cu:1096-1181)."""
    _oo("tdt_peeling_direct_tile_oo", e_curr, rows, columns, row_ptr, support, e_mask, n_mark, in_curr, l, n_cut)


def _check_r_edges(r_edges, E):
    if r_edges.shape[0] < E:
        raise ValueError("r_edges has %d entries, fewer than the %d edges" % (r_edges.shape[0], E))


def _ii(fn, e_curr, rows, columns, r_edges, re_ptr, support, e_mask, n_mark, in_curr, l, n_cut):
    E, args = _peel_common(e_curr, rows, columns, support, e_mask, n_mark, in_curr, (r_edges, re_ptr))
    _check_r_edges(r_edges, E)
    args += [_i32(r_edges, "r_edges"), _i32(re_ptr, "re_ptr"), re_ptr.shape[0]] + _tail(support, e_mask, n_mark,
                                                                                         in_curr)
    args += [int(l)] + ([] if n_cut is None else [int(n_cut)]) + [E, _stream()]
    _call(fn, *args)


def peeling_direct_ii(e_curr, rows, columns, r_edges, re_ptr, support, e_mask, n_mark, in_curr, l):
    """myhpu_extension.cpp:432-446 (kernel.cu:1184-1272): third vertex in the
    in-lists of both ends (r_edges grouped by head, offsets re_ptr)."""
    _ii("tdt_peeling_direct_ii", e_curr, rows, columns, r_edges, re_ptr, support, e_mask, n_mark, in_curr, l, None)


def peeling_direct_tile_ii(e_curr, rows, columns, r_edges, re_ptr, support, e_mask, n_mark, in_curr, l, n_cut):
    """myhpu_extension.cpp:462-476 (kernel.cu:1275-1367)."""
    _ii("tdt_peeling_direct_tile_ii", e_curr, rows, columns, r_edges, re_ptr, support, e_mask, n_mark, in_curr, l,
        n_cut)


def _oi(fn, e_curr, rows, columns, row_ptr, r_edges, re_ptr, support, e_mask, n_mark, in_curr, l, n_cut):
    E, args = _peel_common(e_curr, rows, columns, support, e_mask, n_mark, in_curr, (row_ptr, r_edges, re_ptr))
    _check_r_edges(r_edges, E)
    args += [_i32(row_ptr, "row_ptr"), row_ptr.shape[0], _i32(r_edges, "r_edges"), _i32(re_ptr, "re_ptr"),
             re_ptr.shape[0]] + _tail(support, e_mask, n_mark, in_curr)
    args += [int(l)] + ([] if n_cut is None else [int(n_cut)]) + [E, _stream()]
    _call(fn, *args)


def peeling_direct_oi(e_curr, rows, columns, row_ptr, r_edges, re_ptr, support, e_mask, n_mark, in_curr, l):
    """myhpu_extension.cpp:492-507 (kernel.cu:1370-1457): third vertex in the
    tail's out-list and the head's in-list."""
    _oi("tdt_peeling_direct_oi", e_curr, rows, columns, row_ptr, r_edges, re_ptr, support, e_mask, n_mark, in_curr,
        l, None)


def peeling_direct_tile_oi(e_curr, rows, columns, row_ptr, r_edges, re_ptr, support, e_mask, n_mark, in_curr, l,
                           n_cut):
    """myhpu_extension.cpp:524-540 (kernel.cu:1460-1551)."""
    _oi("tdt_peeling_direct_tile_oi", e_curr, rows, columns, row_ptr, r_edges, re_ptr, support, e_mask, n_mark,
        in_curr, l, n_cut)
