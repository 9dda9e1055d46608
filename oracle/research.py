"""TEST INFRASTRUCTURE ONLY — oracle for the reference's research-variant
operators and the drivers that use them.

* ctypes bindings over the sequential merge walks in ``tdt_oracle.c``
  (``orc_rows_isin_mask``, ``orc_support_affect``, ``orc_peel_op``);
* numpy restatements of the undirected-graph drivers
  ``demo_truss/undirected/truss_undirect_cuda.py`` (symmetric adjacency,
  ``peeling_undirect``) and ``truss_undirect_cuda2.py`` (out- and in-lists,
  ``peeling_direct_oo/ii/oi``), and of the pure-tensor driver
  ``demo_truss/tensor_original/truss_nosavetri_tensor4.py``
  (``segment_isinis_m`` + ``sub_suppport_affect``), step by step.

The reference's OpenMP file has no twin of these operators, so the pin is
through the drivers: each reproduces the sub-rounds the reference's own
``--cuda`` flow recorded for the golden graphs (tests/test_research_ops.py).
Only tests/ may import this module.
"""
import ctypes

import numpy as np

from . import oracle as O

_I32P = O._I32P
_U8P = O._U8P
_ready = False

UNDIRECT, OO, II, OI = 0, 1, 2, 3


def _lib():
    global _ready
    L = O.lib()
    if not _ready:
        i64, i32 = ctypes.c_int64, ctypes.c_int32
        L.orc_rows_isin_mask.argtypes = [_I32P, _I32P, _I32P, _I32P, i64, _U8P, _U8P, ctypes.c_int]
        L.orc_support_affect.argtypes = [_I32P, _I32P, _I32P, i64, _I32P, _U8P, _U8P, _U8P]
        L.orc_peel_op.argtypes = [ctypes.c_int, _I32P, i64, _I32P, _I32P, _I32P, _I32P, _I32P, _I32P, _I32P,
                                  _I32P, _U8P, _U8P, _U8P, i32, i32]
        _ready = True
    return L


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _u8(a):
    return np.ascontiguousarray(a, dtype=np.uint8)


_EMPTY = np.zeros(1, np.int32)


# ---------------------------------------------------------------- operators
def segment_isinis_m(a_columns, a_row_ptr, b_columns, b_row_ptr, mask1, mask2):
    """kernel.cu:687-737; mask1/mask2 are uint8 arrays written in place."""
    _lib().orc_rows_isin_mask(_i32(a_columns), _i32(a_row_ptr), _i32(b_columns), _i32(b_row_ptr),
                              max(len(a_row_ptr) - 1, 0), mask1, mask2, 1)


def segment_isinmm(u_clos, v_clos, uptr, vptr, u_mask, v_mask):
    """kernel.cu:1555-1607."""
    _lib().orc_rows_isin_mask(_i32(u_clos), _i32(uptr), _i32(v_clos), _i32(vptr), max(len(uptr) - 1, 0),
                              u_mask, v_mask, 0)


def sub_suppport_affect(left_nbr, right_nbr, e_curr_rep, support, mask1, mask2, e_affect_mask, l):
    """kernel.cu:739-805 (l unused, as in the reference)."""
    _lib().orc_support_affect(_i32(left_nbr), _i32(right_nbr), _i32(e_curr_rep), len(left_nbr), support,
                              _u8(mask1), _u8(mask2), e_affect_mask)


def peel_op(variant, e_curr, rows, columns, support, e_mask, n_mark, in_curr, l, n_cut=1, row_ptr=None,
            r_edges=None, re_ptr=None, columns_g=None, edges_id_nbr=None):
    """kernel.cu:808-1551.  l is the level as the Python driver passes it; the
    reference's op hands l + 1 to its kernel."""
    def arr(x):
        return _EMPTY if x is None else _i32(x)
    e = _i32(e_curr)
    _lib().orc_peel_op(int(variant), e, len(e), _i32(rows), _i32(columns), arr(row_ptr), arr(r_edges), arr(re_ptr),
                       arr(columns_g), arr(edges_id_nbr), support, _u8(e_mask), n_mark, _u8(in_curr), int(l) + 1,
                       int(n_cut))


# ---------------------------------------------------------------- helpers
def update_row_ptr(keep, row_ptr):
    """truss_undirect_cuda2.py:113-117: per-segment kept counts, re-scanned."""
    vals = np.zeros(len(row_ptr) - 1, np.int32)
    O.segment_add(keep.astype(np.int32), row_ptr, vals)
    return np.concatenate([[0], np.cumsum(vals)]).astype(np.int32)


def _in_list_ptr(rows, cols, r_edges, num_v, n_cut):
    """truss_undirect_cuda2.py:125-136: the in-list offsets (tiled by the
    tail's column tile when n_cut > 1)."""
    if n_cut > 1:
        tiling = num_v // n_cut
        block = rows[r_edges] // (tiling + 1) + cols[r_edges].astype(np.int64) * n_cut
    else:
        block = cols[r_edges].astype(np.int64)
    size_r = np.bincount(block, minlength=num_v * n_cut).astype(np.int32)
    return size_r


def preprocess_direct(rows, cols, rp, num_v, n_cut):
    """truss_undirect_cuda2.py:118-141: the (tiled) out-list offsets, r_edges
    (edge ids stably sorted by head) and their (tiled) offsets re_ptr."""
    rows, cols = _i32(rows), _i32(cols)
    rp_t = O.tiling_row_ptr(rows, cols, num_v, n_cut) if n_cut > 1 else _i32(rp)
    r_edges = np.argsort(cols, kind="stable").astype(np.int32)
    size_r = _in_list_ptr(rows, cols, r_edges, num_v, n_cut)
    re_ptr = np.concatenate([[0], np.cumsum(size_r)]).astype(np.int32)
    return _i32(rp_t), r_edges, re_ptr


def preprocess_undirect(rows, cols, rp, num_v, n_cut_s, n_cut):
    """truss_undirect_cuda.py:80-121: the support-count offsets (tiled by
    n_cut_s) and the symmetric adjacency: slot v*n_cut+k lists the in-neighbours
    of v in tile k, then its out-neighbours in tile k (columns_g), with their
    edge ids (edges_id_nbr) and offsets row_ptr_g."""
    rows, cols = _i32(rows), _i32(cols)
    directed_ptr = O.tiling_row_ptr(rows, cols, num_v, n_cut_s) if n_cut_s > 1 else _i32(rp)
    r_edge = np.argsort(cols, kind="stable").astype(np.int32)
    size_r = _in_list_ptr(rows, cols, r_edge, num_v, n_cut)
    out_ptr = O.tiling_row_ptr(rows, cols, num_v, n_cut) if n_cut > 1 else _i32(rp)
    out_ptr = out_ptr.astype(np.int64)
    ptr_g = out_ptr.copy()
    ptr_g[1:] += np.cumsum(size_r)
    E = len(cols)
    columns_g = np.zeros(2 * E, np.int32)
    edges_id_nbr = np.zeros(2 * E, np.int32)
    in_beg = ptr_g[:-1]
    out_beg = in_beg + size_r
    out_idx = np.concatenate([np.arange(a, b) for a, b in zip(out_beg, ptr_g[1:])]) if E else np.zeros(0, np.int64)
    in_idx = np.concatenate([np.arange(a, b) for a, b in zip(in_beg, out_beg)]) if E else np.zeros(0, np.int64)
    edges_id_nbr[out_idx] = np.arange(E, dtype=np.int32)
    columns_g[out_idx] = cols
    edges_id_nbr[in_idx] = r_edge
    columns_g[in_idx] = rows[r_edge]
    return _i32(directed_ptr), columns_g, edges_id_nbr, ptr_g.astype(np.int32)


def _next_level(support, l, ptr_truss):
    in_curr = support == l
    while not in_curr.any():
        ptr_truss.append(ptr_truss[-1])
        l += 1
        in_curr = support == l
    return l, in_curr


def _peel_loop(support, edges, E_of, peel, compact, compact_threshold):
    """The level / sub-round loop shared by both drivers
    (truss_undirect_cuda.py:165-235, truss_undirect_cuda2.py:193-280)."""
    e_truss, ptr_truss = [], [0]
    l = 1
    if len(support) == 0:              # the reference loops forever here
        return 2, np.zeros(0, np.int32), np.array(ptr_truss, np.int32)
    l, in_curr = _next_level(support, l, ptr_truss)
    e_curr = np.nonzero(in_curr)[0].astype(np.int32)
    e_mask = np.ones(len(support), np.uint8)
    count = 0
    while True:
        while len(e_curr):
            e_truss.append(edges[e_curr])
            n_mark = np.zeros(len(support), np.uint8)
            peel(e_curr, support, e_mask, n_mark, in_curr, l)
            e_mask[e_curr] = 0
            count += len(e_curr)
            in_curr = n_mark.astype(bool)
            e_curr = np.nonzero(n_mark)[0].astype(np.int32)
            if count + len(e_curr) == E_of():
                e_truss.append(edges[e_curr])
                ptr_truss.append(sum(len(x) for x in e_truss))
                return l + 2, np.concatenate(e_truss).astype(np.int32), np.array(ptr_truss, np.int32)
        if count > compact_threshold:
            support, edges = compact(e_mask.astype(bool), support, edges)
            count = 0
            e_mask = np.ones(len(support), np.uint8)
        ptr_truss.append(sum(len(x) for x in e_truss))
        l, in_curr = _next_level(support, l + 1, ptr_truss)
        e_curr = np.nonzero(in_curr)[0].astype(np.int32)


def undirected_truss_direct(rows, cols, rp_t, r_edges, re_ptr, n_cut, compact_threshold=10000000):
    """truss_undirect_cuda2.py:145-280 (undirected_truss): returns
    (kmax, e_truss, ptr_truss).  Edges without triangles are dropped first and
    appear in no level; level l (from 1) holds the edges of truss number l + 2."""
    g = {"rows": _i32(rows).copy(), "cols": _i32(cols).copy(), "rp": _i32(rp_t).copy(),
         "r": _i32(r_edges).copy(), "re": _i32(re_ptr).copy()}
    support = np.zeros(len(g["cols"]), np.int32)
    O.segment_isin2tile(g["rows"], g["cols"], g["rp"], n_cut, support)

    def compact(keep, support, edges):
        g["cols"], g["rows"] = g["cols"][keep], g["rows"][keep]
        g["rp"] = update_row_ptr(keep, g["rp"])
        e_map = np.concatenate([[0], np.cumsum(keep)]).astype(np.int32)
        keep_r = keep[g["r"]]
        g["r"] = e_map[g["r"][keep_r]]
        g["re"] = update_row_ptr(keep_r, g["re"])
        return support[keep], edges[keep]

    support, edges = compact(support != 0, support, np.arange(len(support), dtype=np.int32))

    def peel(e_curr, support, e_mask, n_mark, in_curr, l):
        for v in (OO, II, OI):
            peel_op(v, e_curr, g["rows"], g["cols"], support, e_mask, n_mark, in_curr, l, n_cut,
                    row_ptr=g["rp"], r_edges=g["r"], re_ptr=g["re"])

    return _peel_loop(support, edges, lambda: len(g["cols"]), peel, compact, compact_threshold)


def undirected_truss_undirect(rows, cols, directed_ptr, columns_g, edges_id_nbr, row_ptr_g, n_cut_s, n_cut,
                              compact_threshold=10000000):
    """truss_undirect_cuda.py:125-235 (undirected_truss) over the symmetric
    adjacency from preprocess_undirect; same outputs as
    undirected_truss_direct."""
    g = {"rows": _i32(rows).copy(), "cols": _i32(cols).copy(), "cg": _i32(columns_g).copy(),
         "nbr": _i32(edges_id_nbr).copy(), "pg": _i32(row_ptr_g).copy()}
    support = np.zeros(len(g["cols"]), np.int32)
    O.segment_isin2tile(g["rows"], g["cols"], _i32(directed_ptr), n_cut_s, support)

    def compact(keep, support, edges):
        g["cols"], g["rows"] = g["cols"][keep], g["rows"][keep]
        e_map = np.concatenate([[0], np.cumsum(keep)]).astype(np.int32)
        keep_g = keep[g["nbr"]]
        g["cg"] = g["cg"][keep_g]
        g["nbr"] = e_map[g["nbr"][keep_g]]
        g["pg"] = update_row_ptr(keep_g, g["pg"])
        return support[keep], edges[keep]

    support, edges = compact(support != 0, support, np.arange(len(support), dtype=np.int32))

    def peel(e_curr, support, e_mask, n_mark, in_curr, l):
        peel_op(UNDIRECT, e_curr, g["rows"], g["cols"], support, e_mask, n_mark, in_curr, l, n_cut,
                row_ptr=g["pg"], columns_g=g["cg"], edges_id_nbr=g["nbr"])

    return _peel_loop(support, edges, lambda: len(g["cols"]), peel, compact, compact_threshold)


# ---------------------------------------------------------------- tensor_original driver
def symmetric_csr(rows, cols, num_v):
    """Both directions of every edge, rows sorted by column: the CSRGraph the
    tensor_original driver reads (vertex ids as given)."""
    r = np.concatenate([rows, cols]).astype(np.int64)
    c = np.concatenate([cols, rows]).astype(np.int64)
    order = np.lexsort((c, r))
    r, c = r[order], c[order]
    rp = np.concatenate([[0], np.cumsum(np.bincount(r, minlength=num_v))]).astype(np.int32)
    return rp, c.astype(np.int32)


def _selection(starts, ends):
    """batched_csr_selection_opt2 (helper.py:102-121) on non-empty ranges:
    flat positions and int32 offsets."""
    sizes = (ends - starts).astype(np.int64)
    ptr = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    idx = np.concatenate([np.arange(a, b) for a, b in zip(starts, ends)]) if len(starts) else np.zeros(0, np.int64)
    return idx.astype(np.int64), ptr


def truss_tensor_original(row_ptr, columns, compact_threshold=100000):
    """demo_truss/tensor_original/truss_nosavetri_tensor4.py:27-196
    (truss_deposs) over a symmetric CSR: returns (e_truss, ptr_truss) over the
    undirected edges u < v in CSR order.  As in the reference, the edges of
    the last sub-round are not appended to e_truss (:147-152 stops first)."""
    row_ptr = _i32(row_ptr).astype(np.int64)
    columns = _i32(columns).copy()
    V = len(row_ptr) - 1
    row_indice_g = np.repeat(np.arange(V, dtype=np.int32), np.diff(row_ptr))
    mask = row_indice_g < columns
    row_indice = row_indice_g[mask]
    cols_u = columns[mask]
    Eu = len(cols_u)
    e_truss, ptr_truss = [], [0]
    e_mask = np.ones(Eu, bool)
    edges_id = np.arange(Eu, dtype=np.int32)
    edges_id_nbr = np.arange(len(columns), dtype=np.int32)
    edges_id_nbr[mask] = edges_id
    sorted_indices = np.argsort(columns[~mask], kind="stable")
    temp = np.zeros(Eu, np.int32)
    temp[sorted_indices] = edges_id
    edges_id_nbr[~mask] = temp
    direc = np.zeros(V, np.int32)
    O.segment_add(mask.astype(np.int32), row_ptr.astype(np.int32), direc)
    direc_rp = np.concatenate([[0], np.cumsum(direc)]).astype(np.int32)
    support = np.zeros(Eu, np.int32)
    O.segment_isin2tile(row_indice, cols_u, direc_rp, 1, support)
    e_mask[edges_id[support == 0]] = False
    if not e_mask.any():
        return np.zeros(0, np.int32), np.array(ptr_truss, np.int32)
    keep = e_mask[edges_id_nbr]
    edges_id_nbr = edges_id_nbr[keep]
    columns = columns[keep]
    sizes = np.zeros(V, np.int32)
    O.segment_add(keep.astype(np.int32), row_ptr.astype(np.int32), sizes)
    row_ptr = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    l = 1
    e_curr = edges_id[support == l]
    while len(e_curr) == 0:
        ptr_truss.append(sum(len(x) for x in e_truss))
        l += 1
        e_curr = edges_id[support == l]
    e_del = 0
    columns = np.concatenate([columns, [-1]]).astype(np.int32)
    n_out = lambda: sum(len(x) for x in e_truss)
    while True:
        e_truss.append(edges_id[e_curr])
        left, s_ptr = _selection(row_ptr[row_indice[e_curr]], row_ptr[row_indice[e_curr] + 1])
        right, e_ptr = _selection(row_ptr[cols_u[e_curr]], row_ptr[cols_u[e_curr] + 1])
        m1 = e_mask[edges_id_nbr[left]]
        m2 = e_mask[edges_id_nbr[right]]
        left = left.copy()
        right = right.copy()
        left[~m1] = -1
        right[~m2] = -1
        mk1 = np.zeros(len(left), np.uint8)
        mk2 = np.zeros(len(right), np.uint8)
        segment_isinis_m(columns[left], s_ptr, columns[right], e_ptr, mk1, mk2)
        mk1, mk2 = mk1.astype(bool), mk2.astype(bool)
        left_nbr = edges_id_nbr[left[mk1]]
        right_nbr = edges_id_nbr[right[mk2]]
        if len(left_nbr) == 0 or len(right_nbr) == 0:
            e_mask[e_curr] = False
            e_curr = left_nbr
        else:
            values = np.zeros(len(e_ptr) - 1, np.int32)
            O.segment_add(mk2.astype(np.int32), e_ptr, values)
            e_curr_rep = np.repeat(e_curr, values)
            s1 = (support[left_nbr] > l).astype(np.uint8)
            s2 = (support[right_nbr] > l).astype(np.uint8)
            affect = np.zeros(len(e_mask), np.uint8)
            sub_suppport_affect(left_nbr, right_nbr, e_curr_rep, support, s1, s2, affect, l)
            e_del += len(e_curr)
            e_mask[e_curr] = False
            e_aff = np.nonzero(affect)[0]
            e_curr = e_aff[support[e_aff] <= l].astype(np.int32)
        if int(e_mask.sum()) == len(e_curr):
            ptr_truss.append(n_out())
            break
        if e_del >= compact_threshold:
            keep = e_mask[edges_id_nbr]
            edges_id_nbr = edges_id_nbr[keep]
            columns = np.concatenate([columns[:-1][keep], [-1]]).astype(np.int32)
            sizes = np.zeros(V, np.int32)
            O.segment_add(keep.astype(np.int32), row_ptr.astype(np.int32), sizes)
            row_ptr = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
            e_del = 0
            idx = np.nonzero(e_mask)[0]
            edges_id, support, cols_u, row_indice = edges_id[idx], support[idx], cols_u[idx], row_indice[idx]
            remap = np.zeros(len(e_mask), np.int32)
            remap[idx] = np.arange(len(idx), dtype=np.int32)
            e_curr = remap[e_curr]
            edges_id_nbr = remap[edges_id_nbr]
            e_mask = np.ones(len(idx), bool)
        if len(e_curr) == 0:
            ptr_truss.append(n_out())
            l += 1
            e_curr = np.nonzero(support == l)[0].astype(np.int32)
            while len(e_curr) == 0:
                ptr_truss.append(n_out())
                l += 1
                e_curr = np.nonzero(support == l)[0].astype(np.int32)
    e = np.concatenate(e_truss).astype(np.int32) if e_truss else np.zeros(0, np.int32)
    return e, np.array(ptr_truss, np.int32)
