"""TEST INFRASTRUCTURE ONLY — the oracle's Python face.

CPU restatement of the reference's truss-decomposition path:

* ctypes bindings over ``tdt_oracle.c`` (operators + the ``k_truss`` drivers);
* numpy restatements of the preprocessing (``Graph.read_edgelist``,
  ``CSRCOO.edge_list_to_Graph``, ``csr_to_tilingcsr``);
* the k-truss search driver (``ktruss_search/ktruss_cuda.py:383-463``);
* optional bindings over the reference's own OpenMP operators built into
  ``oracle/_ref`` (``ref_ops()``), used to pin the restatement.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs may import
this module.  The product package never does.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_I32P = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_U8P = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_I64P = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        path = _build.ORACLE_SO
        if not os.path.exists(path):
            path = _build.build_oracle()
        L = ctypes.CDLL(path)
        i64, i32 = ctypes.c_int64, ctypes.c_int32
        L.orc_segment_add.argtypes = [_I32P, _I32P, _I32P, i64]
        L.orc_segment_isin2tile.argtypes = [_I32P, _I32P, _I32P, i32, _I32P, i64]
        L.orc_segment_isin2tile_k.argtypes = [_I32P, _I32P, _I32P, i32, i32, _I32P, i64]
        L.orc_all_affected_support_tile.argtypes = [_I32P, i64, _I32P, _I32P, _I32P, i32, _U8P, i32, _U8P, _I32P]
        L.orc_all_affected_support_tilenot.argtypes = [_I32P, i64, _I32P, _I32P, _I32P, i32, _U8P, i32, _U8P, _I32P]
        L.orc_all_affected_support_tilenotwin.argtypes = [_I32P, i64, _I32P, _I32P, _I32P, i32, _U8P, i32, _U8P,
                                                          _I32P, i32, _U8P, _I32P, _I32P]
        L.orc_sub_affected_support_tile.argtypes = [_I32P, _I32P, _I32P, i32, _U8P, _I32P, i64]
        L.orc_k_truss.argtypes = [_I32P, _I32P, _I32P, i64, i64, i32, i32, _I32P,
                                  ctypes.POINTER(i64), _I32P, i64, ctypes.POINTER(i64)]
        L.orc_k_truss.restype = i32
        L.orc_truss_from_levels.argtypes = [_I32P, _I32P, i64, i64, _I32P]
        L.orc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def ref_ops():
    """ctypes handle on the reference's own OpenMP operators, or None."""
    global _ref
    if _ref is None:
        path = _build.REF_SO if os.path.exists(_build.REF_SO) else _build.build_ref()
        if path is None or not os.path.exists(path):
            return None
        L = ctypes.CDLL(path)
        i32 = ctypes.c_int
        L.ref_segment_add.argtypes = [_I32P, _I32P, _I32P, i32]
        L.ref_segment_isin2.argtypes = [_I32P, _I32P, _I32P, _I32P, i32]
        L.ref_segment_isin2tile.argtypes = [_I32P, _I32P, _I32P, i32, _I32P, i32]
        L.ref_all_affected_support.argtypes = [_I32P, _I32P, _I32P, _I32P, _U8P, i32, _U8P, _I32P, i32]
        L.ref_all_affected_support_tile.argtypes = [_I32P, _I32P, _I32P, _I32P, i32, _U8P, i32, _U8P, _I32P, i32]
        _ref = L
    return _ref


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _u8(a):
    return np.ascontiguousarray(a, dtype=np.uint8)


# ---------------------------------------------------------------- operators
def segment_add(col_indices, col_ptr, out):
    lib().orc_segment_add(_i32(col_indices), _i32(col_ptr), out, out.shape[0])


def segment_isin2tile(rows, cols, rp, n_cut, out):
    lib().orc_segment_isin2tile(_i32(rows), _i32(cols), _i32(rp), int(n_cut), out, out.shape[0])


def segment_isin2tile_k(rows, cols, rp, n_cut, k, out):
    lib().orc_segment_isin2tile_k(_i32(rows), _i32(cols), _i32(rp), int(n_cut), int(k), out, out.shape[0])


def all_affected_support_tile(e_affect, rows, cols, rp, n_cut, mark, l, n_mark, out):
    ea = _i32(e_affect)
    lib().orc_all_affected_support_tile(ea, ea.shape[0], _i32(rows), _i32(cols), _i32(rp), int(n_cut),
                                        _u8(mark), int(l), n_mark, out)


def all_affected_support_tilenot(e_affect, rows, cols, rp, n_cut, mark, l, n_mark, out):
    ea = _i32(e_affect)
    lib().orc_all_affected_support_tilenot(ea, ea.shape[0], _i32(rows), _i32(cols), _i32(rp), int(n_cut),
                                           _u8(mark), int(l), n_mark, out)


def all_affected_support_tilenotwin(e_affect, rows, cols, rp, n_cut, mark, l, n_mark, out,
                                    windows_high, in_win, buff_index, buf_size):
    ea = _i32(e_affect)
    lib().orc_all_affected_support_tilenotwin(ea, ea.shape[0], _i32(rows), _i32(cols), _i32(rp), int(n_cut),
                                              _u8(mark), int(l), n_mark, out, int(windows_high), in_win,
                                              buff_index, buf_size)


def sub_affected_support_tile(rows, cols, rp, n_cut, mark, out):
    lib().orc_sub_affected_support_tile(_i32(rows), _i32(cols), _i32(rp), int(n_cut), _u8(mark), out,
                                        out.shape[0])


def support(rows, cols, rp, n_cut=1):
    out = np.zeros(len(cols), np.int32)
    segment_isin2tile(rows, cols, rp, n_cut, out)
    return out


# ---------------------------------------------------------------- drivers
def k_truss(rows, cols, rp_tiled, num_v, n_cut, cpu_flow=False):
    """singlegpu_truss.py:67-158 (cpu_flow=False) / test/truss_setup.py:61-154
    (cpu_flow=True).  Returns (kmax, e_truss, ptr_truss, truss_per_edge)."""
    rows, cols, rp = _i32(rows), _i32(cols), _i32(rp_tiled)
    E = cols.shape[0]
    e_truss = np.zeros(max(E, 1), np.int32)
    cap = E + 8
    ptr = np.zeros(cap, np.int32)
    n_et = ctypes.c_int64(0)
    n_ptr = ctypes.c_int64(0)
    kmax = lib().orc_k_truss(rows, cols, rp, int(num_v), int(E), int(n_cut), int(bool(cpu_flow)),
                             e_truss, ctypes.byref(n_et), ptr, cap, ctypes.byref(n_ptr))
    if kmax < 0:
        raise RuntimeError("oracle k_truss: level table overflow")
    e_truss = e_truss[:n_et.value].copy()
    ptr = ptr[:n_ptr.value].copy()
    truss = np.zeros(max(E, 1), np.int32)
    lib().orc_truss_from_levels(e_truss if e_truss.size else np.zeros(1, np.int32), ptr, ptr.shape[0], E, truss)
    return int(kmax), e_truss, ptr, truss[:E]


def ktruss_search(rows, cols, rp_tiled, num_v, n_cut, k):
    """ktruss_search/ktruss_cuda.py:383-463 with l = k - 2 (:507).  The graph
    arrays are copied; returns the surviving edges as (rows, cols) pairs of
    the compacted graph, exactly as the reference's e_rest indexes them."""
    l = int(k) - 2
    rows, cols, rp = _i32(rows).copy(), _i32(cols).copy(), _i32(rp_tiled).copy()
    E = cols.shape[0]
    sup = np.zeros(E, np.int32)
    segment_isin2tile_k(rows, cols, rp, n_cut, l, sup)           # support_computing_k (:347-355)
    if l == 1:
        e_rest = np.nonzero(sup >= 1)[0]                          # :388-390
        return rows[e_rest], cols[e_rest]
    mask = sup < l                                               # :403
    e_del = np.nonzero(mask)[0]
    ed_count = e_del.shape[0]
    while e_del.shape[0] != 0 and ed_count != sup.shape[0]:       # :406
        if ed_count >= sup.shape[0] / 32:                         # compaction (:407-420)
            f_mask = ~mask
            e_rest = np.nonzero(f_mask)[0]
            cols = cols[e_rest]
            rows = rows[e_rest]
            vals = np.zeros(rp.shape[0] - 1, np.int32)
            segment_add(f_mask.astype(np.int32), rp, vals)
            rp = np.concatenate([[0], np.cumsum(vals)]).astype(np.int32)
            sup = support(rows, cols, rp, n_cut)                  # full support (:416)
            mask = sup < l
            e_del = np.nonzero(mask)[0].astype(np.int32)
            ed_count = e_del.shape[0]
        else:                                                     # affected subgraph (:424-456)
            pa = np.unique(np.concatenate([rows[e_del], cols[e_del]]))
            mask_v = np.zeros(num_v + 1, bool)
            mask_v[pa] = True
            mask_a = mask_v[cols]                                 # index -1 -> mask_v[num_v]
            p_c = np.concatenate([np.arange(rp[p * n_cut], rp[p * n_cut + n_cut]) for p in pa]) \
                if pa.size else np.zeros(0, np.int64)
            mask_a[p_c] = cols[p_c] != -1
            e_affect = np.nonzero(mask_a)[0].astype(np.int32)
            sub_rows = rows[e_affect]
            sub_cols = cols[e_affect]
            sub_rp = np.zeros(rp.shape[0] - 1, np.int32)
            segment_add(mask_a.astype(np.int32), rp, sub_rp)
            sub_rp = np.concatenate([[0], np.cumsum(sub_rp)]).astype(np.int32)
            sub_sup = sup[e_affect].copy()
            mark = mask[e_affect]
            sub_affected_support_tile(sub_rows, sub_cols, sub_rp, n_cut, mark, sub_sup)
            sup[e_affect] = sub_sup
            s_mask = sub_sup < l
            cols[e_del] = -1
            e_del = e_affect[s_mask & (~mark)]
            mask[e_del] = True
            ed_count += e_del.shape[0]
    e_rest = np.nonzero(~mask)[0]
    return rows[e_rest], cols[e_rest]


# ---------------------------------------------------------------- preprocessing
def read_edgelist_arrays(pairs, stable=True):
    """src/type/Graph_Truss.py:177-213 on an int32 [M,2] array already read
    from the file: drop self-loops (:188), dedup unordered pairs keeping the
    first occurrence's orientation (:200-202), rank vertices by degree
    (:209-211).  stable=True breaks degree ties by vertex id (the (degree, id)
    rank); stable=False uses numpy's default argsort exactly as the
    reference does."""
    arr = np.asarray(pairs, dtype=np.int32).reshape(-1, 2)
    arr = arr[arr[:, 0] != arr[:, 1]]
    _, idx = np.unique(np.sort(arr, axis=1), return_index=True, axis=0)
    starts = arr[idx, 0]
    ends = arr[idx, 1]
    vertices, counts = np.unique(np.concatenate((starts, ends)), return_counts=True)
    order = np.argsort(counts, kind="stable") if stable else np.argsort(counts)
    return starts, ends, vertices[order]


def edge_list_to_csr(starts, ends, vertices):
    """src/type/CSRCOO.py:128-162 + counter_sort (:169-177): relabel by rank,
    orient low->high, CSR by row with columns sorted within a row.  Returns
    (rows, columns, row_ptr) int32."""
    V = vertices.shape[0]
    order = np.argsort(vertices, kind="stable")
    sv = vertices[order]
    s = order[np.searchsorted(sv, starts)].astype(np.int64)
    e = order[np.searchsorted(sv, ends)].astype(np.int64)
    lo = np.minimum(s, e)
    hi = np.maximum(s, e)
    row_ptr = np.concatenate([[0], np.cumsum(np.bincount(lo, minlength=V))]).astype(np.int32)
    perm = np.lexsort((hi, lo))
    return lo[perm].astype(np.int32), hi[perm].astype(np.int32), row_ptr


def preprocess(pairs, stable=True):
    s, e, v = read_edgelist_arrays(pairs, stable)
    rows, cols, rp = edge_list_to_csr(s, e, v)
    return rows, cols, rp, v


def tiling_row_ptr(rows, cols, num_v, n_cut):
    """csr_to_tilingcsr (singlegpu_truss.py:160-169): tile j of vertex u holds
    the out-neighbours w with w // (V // n_cut + 1) == j."""
    if n_cut == 1:
        rp = np.zeros(num_v + 1, np.int64)
        np.add.at(rp, np.asarray(rows, np.int64) + 1, 1)
        return np.cumsum(rp).astype(np.int32)
    tiling = num_v // n_cut
    block = np.asarray(cols, np.int64) // (tiling + 1) + np.asarray(rows, np.int64) * n_cut
    cnt = np.bincount(block, minlength=num_v * n_cut)
    return np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)


def undirected_truss_map(rows, cols, truss, vertices):
    """{(min(orig_u, orig_v), max(...)): truss} — the orientation-invariant
    key used to compare results across different vertex rankings."""
    ou = vertices[np.asarray(rows)]
    ov = vertices[np.asarray(cols)]
    lo = np.minimum(ou, ov)
    hi = np.maximum(ou, ov)
    return {(int(a), int(b)): int(t) for a, b, t in zip(lo, hi, truss)}


def num_threads():
    return int(lib().orc_num_threads())
