"""The reference's `--cuda` driver flow on top of the drop-in operators.

The algorithm layer of singlegpu_truss.py (support_computing :38-45,
all_affect_support_not :54-58, update_row_ptr :60-64, k_truss :67-158) and
the CPU-capable flow of demo_truss/test/truss_setup.py (:61-154), written
against :mod:`tdtdecomposition_gb300.trusstensor`.  It keeps the reference's
host-driven sub-round loop on purpose: it is the compatibility path that
shows the operators behave as drop-ins inside the reference's own control
flow.  The device-resident replacement of this loop is
:func:`tdtdecomposition_gb300.truss.truss_decompose`.

Unlike the reference, k_truss returns the peel order as well
(e_truss, ptr_truss); singlegpu_truss.py:158 returns only kmax and times.
"""
import torch

from . import trusstensor as tt


def support_computing(sub_rows, sub_columns, tiling_row_ptr, n_cut):
    support = torch.zeros(sub_columns.shape[0], dtype=torch.int32, device=sub_columns.device)
    if n_cut > 1:
        tt.segment_isin2tile(sub_rows, sub_columns, tiling_row_ptr, n_cut, support)
    else:
        tt.segment_isin2(sub_rows, sub_columns, tiling_row_ptr, support)
    return support


def all_affect_support(e_affect, graph, n_cut, mask, l, n_mark, support):
    if n_cut > 1:
        tt.sub_AllAffectedSupport_tile(e_affect, graph.rows, graph.columns, graph.row_ptr, n_cut, mask, l, n_mark,
                                       support)
    else:
        tt.sub_AllAffectedSupport(e_affect, graph.rows, graph.columns, graph.row_ptr, mask, l, n_mark, support)


def all_affect_support_not(e_affect, graph, n_cut, mask, l, n_mark, support):
    if n_cut > 1:
        tt.sub_AllAffectedSupport_tilenot(e_affect, graph.rows, graph.columns, graph.row_ptr, n_cut, mask, l,
                                          n_mark, support)
    else:
        tt.sub_AllAffectedSupport_not(e_affect, graph.rows, graph.columns, graph.row_ptr, mask, l, n_mark,
                                      support)


def update_row_ptr(e_mask, row_ptr):
    values = torch.zeros(row_ptr.shape[0] - 1, dtype=torch.int32, device=row_ptr.device)
    tt.segment_add(e_mask.int(), row_ptr, values)
    return torch.cat([torch.zeros(1, dtype=torch.int32, device=row_ptr.device),
                      values.cumsum(0, dtype=torch.int32)])


def _batched_csr_selection(starts, ends):
    """Flat positions of all [starts[i], ends[i]) ranges (helper.py:102-121)."""
    sizes = (ends - starts).to(torch.int64)
    total = int(sizes.sum())
    if total == 0:
        return torch.zeros(0, dtype=torch.int64, device=starts.device)
    seg = torch.repeat_interleave(torch.arange(sizes.shape[0], device=starts.device), sizes)
    first = torch.cumsum(sizes, 0) - sizes
    return starts.to(torch.int64)[seg] + (torch.arange(total, device=starts.device) - first[seg])


def _csr_selection_ptr(starts, ends):
    """batched_csr_selection_opt (helper.py:87-101): flat positions of all
    [starts[i], ends[i]) ranges and their int32 offsets."""
    sizes = (ends - starts).to(torch.int64).clamp_(min=0)
    ptr = torch.zeros(sizes.shape[0] + 1, dtype=torch.int32, device=starts.device)
    ptr[1:] = torch.cumsum(sizes, 0).to(torch.int32)
    return _batched_csr_selection(starts, starts + sizes), ptr


def _rows_of(row_ptr, v, n_cut):
    """Whole-row ranges of vertices v in a (tiled) row_ptr."""
    rp = row_ptr.to(torch.int64)
    v = v.to(torch.int64)
    return rp[v * n_cut], rp[v * n_cut + n_cut]


# ------------------------------------------------------------------ fusion ablation ("before" ops)
def support_computing_before(sub_rows, sub_columns, tiling_row_ptr, n_cut):
    """fusionexperiental.py:24-46: the unfused support count the reference
    times as "ComputeSup" against segment_isin2 ("ComputeSup+").  Every edge
    (u, v) gathers N+(u) and N+(v), segment_isinmm marks their common
    neighbours, and three separate passes count the triangles of (u, v),
    (u, w) and (v, w).  The reference calls it with n_cut = 1 and indexes
    row_ptr[u], row_ptr[u + 1]; whole rows (row_ptr[u * n_cut] ..
    row_ptr[u * n_cut + n_cut]) are the same there and stay right for tiled
    offsets.  Same result as support_computing."""
    E = sub_columns.shape[0]
    support = torch.zeros(E, dtype=torch.int32, device=sub_columns.device)
    I_u, uptr = _csr_selection_ptr(*_rows_of(tiling_row_ptr, sub_rows, n_cut))
    I_v, vptr = _csr_selection_ptr(*_rows_of(tiling_row_ptr, sub_columns, n_cut))
    M_u = torch.zeros(I_u.shape[0], dtype=torch.bool, device=support.device)
    M_v = torch.zeros(I_v.shape[0], dtype=torch.bool, device=support.device)
    tt.segment_isinmm(sub_columns[I_u], sub_columns[I_v], uptr, vptr, M_u, M_v)
    tt.segment_add(M_u.int(), uptr, support)
    I_uw, ct = torch.unique(I_u[M_u], return_counts=True)
    support[I_uw] += ct.to(torch.int32)
    I_vw, ct = torch.unique(I_v[M_v], return_counts=True)
    support[I_vw] += ct.to(torch.int32)
    return support


def all_affect_support_not_before(e_affect, graph, n_cut, mask, l, n_mark, support):
    """fusionexperiental.py:48-67: the unfused peel update (the reference
    defines it next to its timed support phase and never reaches it).  For
    each affected edge (u, v), segment_isinmm pairs N+(u) with N+(v); a
    triangle whose (u, w) column is live and whose three edges are not all in
    `mask` is destroyed: all three edges lose one, and the touched edges in
    `mask` that end at or below l are set in n_mark.  Affected edges whose
    column is already -1 (peeled) carry no triangle here; the reference would
    index row_ptr[-1] for them.  Same n_mark as all_affect_support_not."""
    e_affect = e_affect.to(torch.int64)
    e_affect = e_affect[graph.columns[e_affect] >= 0]
    U = graph.rows[e_affect]
    V = graph.columns[e_affect]
    I_u, uptr = _csr_selection_ptr(*_rows_of(graph.row_ptr, U, n_cut))
    I_v, vptr = _csr_selection_ptr(*_rows_of(graph.row_ptr, V, n_cut))
    M_u = torch.zeros(I_u.shape[0], dtype=torch.bool, device=support.device)
    M_v = torch.zeros(I_v.shape[0], dtype=torch.bool, device=support.device)
    tt.segment_isinmm(graph.columns[I_u], graph.columns[I_v], uptr, vptr, M_u, M_v)
    sizes = torch.zeros(e_affect.shape[0], dtype=torch.int32, device=support.device)
    tt.segment_add(M_u.int(), uptr, sizes)
    I_uv = torch.repeat_interleave(e_affect, sizes.to(torch.int64))
    I_uw = I_u[M_u]
    I_vw = I_v[M_v]
    M_tri = (graph.columns[I_uw] > 0) & (~(mask[I_uv] & mask[I_uw] & mask[I_vw]))
    I_e = torch.cat([I_uv[M_tri], I_uw[M_tri], I_vw[M_tri]])
    I_ue, counts = torch.unique(I_e, return_counts=True)
    support[I_ue] -= counts.to(torch.int32)
    n_mark[I_ue] = mask[I_ue] & (support[I_ue] <= l)
    return n_mark, support


def k_truss(graph, n_cut, num_v, cpu_flow=False, compact_threshold=1000000, fused=True, fused_support=None,
            fused_update=None):
    """singlegpu_truss.py:67-158 (cpu_flow=False, peel update = *_not) or
    test/truss_setup.py:61-154 (cpu_flow=True, peel update = sub_AllAffectedSupport*).
    fused=False runs the fusion experiment's unfused operators instead
    (support_computing_before, all_affect_support_not_before;
    fusionexperiental.py:24-67) with the same results; fused_support /
    fused_update choose each half on its own (the four columns of the
    reference's ablation: TDT-origin, +Comp, +Update, +both).
    Mutates graph like the reference.  Returns (kmax, e_truss, ptr_truss)."""
    dev = graph.device
    fused_support = fused if fused_support is None else fused_support
    fused_update = fused if fused_update is None else fused_update
    if fused_support:
        support = support_computing(graph.rows, graph.columns, graph.row_ptr, n_cut)
    else:
        support = support_computing_before(graph.rows, graph.columns, graph.row_ptr, n_cut)
    e_truss = torch.zeros(0, dtype=torch.int32, device=dev)
    ptr_truss = [0]
    l = 1
    edges = torch.arange(graph.columns.shape[0], dtype=torch.int32, device=dev)
    e_mask = support.bool()
    edges = edges[e_mask]
    support = support[e_mask]
    graph.columns = graph.columns[e_mask]
    graph.rows = graph.rows[e_mask]
    graph.row_ptr = update_row_ptr(e_mask, graph.row_ptr)
    if graph.columns.shape[0] == 0:  # the reference loops forever here (no triangle)
        return 2, e_truss, torch.tensor(ptr_truss, dtype=torch.int32)
    e_curr = torch.where(support == l)[0]
    while e_curr.shape[0] == 0:
        ptr_truss.append(ptr_truss[-1])
        l += 1
        e_curr = torch.where(support == l)[0]
    peeled = 0
    e_mask = (torch.zeros if cpu_flow else torch.ones)(graph.columns.shape[0], dtype=torch.bool, device=dev)
    while True:
        e_truss = torch.cat([e_truss, edges[e_curr]])
        p = torch.unique(graph.rows[e_curr])
        mask_v = torch.zeros(num_v, dtype=torch.bool, device=dev)
        mask_v[p] = True
        mask = mask_v[graph.columns.long()]  # index -1 reads the last vertex, as in Python
        p_c = _batched_csr_selection(graph.row_ptr[p * n_cut], graph.row_ptr[p * n_cut + n_cut])
        mask[p_c] = ~e_mask[p_c] if cpu_flow else e_mask[p_c]
        e_affect = torch.where(mask)[0].to(torch.int32)
        e_mask[e_curr] = cpu_flow
        n_mark = torch.zeros(graph.columns.shape[0], dtype=torch.bool, device=dev)
        if cpu_flow:
            all_affect_support(e_affect, graph, n_cut, e_mask, l, n_mark, support)
        elif fused_update:
            all_affect_support_not(e_affect, graph, n_cut, e_mask, l, n_mark, support)
        else:
            all_affect_support_not_before(e_affect, graph, n_cut, e_mask, l, n_mark, support)
        graph.columns[e_curr] = -1
        peeled += e_curr.shape[0]
        if peeled > compact_threshold:
            keep = ~e_mask if cpu_flow else e_mask
            support = support[keep]
            graph.columns = graph.columns[keep]
            graph.rows = graph.rows[keep]
            edges = edges[keep]
            graph.row_ptr = update_row_ptr(keep, graph.row_ptr)
            peeled = 0
            e_curr = torch.where(support <= l)[0]
            e_mask = (torch.zeros if cpu_flow else torch.ones)(graph.columns.shape[0], dtype=torch.bool, device=dev)
        else:
            e_curr = torch.where(n_mark)[0]
            e_curr = e_curr[support[e_curr] <= l]
        if peeled + e_curr.shape[0] == graph.columns.shape[0]:
            e_truss = torch.cat([e_truss, edges[e_curr]])
            ptr_truss.append(e_truss.shape[0])
            break
        if e_curr.shape[0] == 0:
            ptr_truss.append(e_truss.shape[0])
            l += 1
            e_curr = torch.where(support == l)[0]
            while e_curr.shape[0] == 0:
                ptr_truss.append(ptr_truss[-1])
                l += 1
                e_curr = torch.where(support == l)[0]
    return l + 2, e_truss, torch.tensor(ptr_truss, dtype=torch.int32)


def all_affect_support_not_win(e_affect, graph, n_cut, mask, l, n_mark, support, windows_high, in_windows_mask,
                               buff_index, buf_size):
    """multigpu_truss_pre4.py:62-66 (the pybind names *_notwin)."""
    if n_cut > 1:
        tt.sub_AllAffectedSupport_tilenotwin(e_affect, graph.rows, graph.columns, graph.row_ptr, n_cut, mask, l,
                                             n_mark, support, windows_high, in_windows_mask, buff_index, buf_size)
    else:
        tt.sub_AllAffectedSupport_notwin(e_affect, graph.rows, graph.columns, graph.row_ptr, mask, l, n_mark,
                                         support, windows_high, in_windows_mask, buff_index, buf_size)


def k_truss_windowed(graph, n_cut, num_v, windows_skip=16, compact_threshold=10000000):
    """The support-window flow of demo_truss/multigpu_truss_pre4.py:75-199.

    Edges whose support lies in the window [l, windows_high) are kept in a
    buffer (buff_index[:buf_size]); the *_notwin peel update appends every edge
    whose support falls into the window, so a new level's frontier is found in
    the buffer instead of all edges, and the window moves up by windows_skip
    levels when l reaches its top.  Mutates graph like the reference.
    Returns (kmax, e_truss, ptr_truss): ptr_truss[j]..ptr_truss[j+1] are the
    edges of level j+1 (truss number j+3); support-0 edges are left out.
    Within a sub-round the order of e_truss follows the buffer, whose appends
    are concurrent, so only the per-level sets are deterministic."""
    dev = graph.device
    support = support_computing(graph.rows, graph.columns, graph.row_ptr, n_cut)
    e_truss = torch.zeros(0, dtype=torch.int32, device=dev)
    ptr_truss = [0]
    l = 1
    edges = torch.arange(graph.columns.shape[0], dtype=torch.int32, device=dev)
    e_mask = support.bool()
    edges = edges[e_mask]
    support = support[e_mask]
    graph.columns = graph.columns[e_mask]
    graph.rows = graph.rows[e_mask]
    graph.row_ptr = update_row_ptr(e_mask, graph.row_ptr)
    E = graph.columns.shape[0]
    if E == 0:  # the reference loops forever here (no triangle)
        return 2, e_truss, torch.tensor(ptr_truss, dtype=torch.int32)
    edges_curr = torch.arange(E, dtype=torch.int32, device=dev)
    buff_index = torch.zeros(E, dtype=torch.int32, device=dev)
    buf_size = torch.zeros(1, dtype=torch.int32, device=dev)
    windows_high = l + windows_skip

    def fill_window(lo):
        nonlocal in_windows_mask
        in_windows_mask = (support >= lo) & (support < windows_high)
        buff = edges_curr[in_windows_mask]
        buf_size[0] = buff.shape[0]
        buff_index[: buff.shape[0]] = buff

    def frontier():
        b = buff_index[: int(buf_size[0])].long()
        return b[support[b] == l].to(torch.int32)

    in_windows_mask = None
    fill_window(0)
    e_curr = frontier()

    def next_level():
        nonlocal l, windows_high, e_curr
        e = e_curr
        while e.shape[0] == 0:
            ptr_truss.append(ptr_truss[-1])
            l += 1
            if l == windows_high:
                windows_high = l + windows_skip
                fill_window(l)
            e = frontier()
        e_curr = e

    next_level()
    peeled = 0
    e_mask = torch.ones(E, dtype=torch.bool, device=dev)
    while True:
        e_truss = torch.cat([e_truss, edges[e_curr.long()]])
        p = torch.unique(graph.rows[e_curr.long()])
        mask_v = torch.zeros(num_v, dtype=torch.bool, device=dev)
        mask_v[p] = True
        mask = mask_v[graph.columns.long()]  # index -1 reads the last vertex, as in Python
        p_c = _batched_csr_selection(graph.row_ptr[p * n_cut], graph.row_ptr[p * n_cut + n_cut])
        mask[p_c] = e_mask[p_c]
        e_affect = edges_curr[mask]
        e_mask[e_curr.long()] = False
        n_mark = torch.zeros(graph.columns.shape[0], dtype=torch.bool, device=dev)
        all_affect_support_not_win(e_affect, graph, n_cut, e_mask, l, n_mark, support, windows_high,
                                   in_windows_mask, buff_index, buf_size)
        graph.columns[e_curr.long()] = -1
        peeled += e_curr.shape[0]
        if peeled > compact_threshold:
            support = support[e_mask]
            graph.columns = graph.columns[e_mask]
            graph.rows = graph.rows[e_mask]
            edges = edges[e_mask]
            graph.row_ptr = update_row_ptr(e_mask, graph.row_ptr)
            in_windows_mask = in_windows_mask[e_mask]
            peeled = 0
            edges_curr = torch.arange(graph.columns.shape[0], dtype=torch.int32, device=dev)
            buff_index = torch.zeros(graph.columns.shape[0], dtype=torch.int32, device=dev)
            buff = edges_curr[in_windows_mask]
            buf_size[0] = buff.shape[0]
            buff_index[: buff.shape[0]] = buff
            n_mark = n_mark[e_mask]
            e_mask = torch.ones(graph.columns.shape[0], dtype=torch.bool, device=dev)
        e_curr = edges_curr[n_mark]
        if peeled + e_curr.shape[0] == graph.columns.shape[0]:
            e_truss = torch.cat([e_truss, edges[e_curr.long()]])
            ptr_truss.append(e_truss.shape[0])
            break
        if e_curr.shape[0] == 0:
            ptr_truss.append(e_truss.shape[0])
            l += 1
            if l == windows_high:
                windows_high = l + windows_skip
                fill_window(l)
            e_curr = frontier()
            next_level()
    return l + 2, e_truss, torch.tensor(ptr_truss, dtype=torch.int32)


# ------------------------------------------------------------------ undirected-graph drivers
# demo_truss/undirected/truss_undirect_cuda.py and truss_undirect_cuda2.py: the
# same level / sub-round peel as k_truss, but every current edge removes its
# triangles itself through the oriented (peeling_direct_oo/ii/oi) or the
# symmetric (peeling_undirect) update, so no affected-edge gather is needed.
# Edges in no triangle are dropped before the peel and appear in no level;
# level l (from 1) holds the edges of truss number l + 2.  The input graph is
# left untouched.

def _in_list_sizes(rows, cols, r_edges, num_v, n_cut):
    if n_cut > 1:
        block = rows[r_edges].to(torch.int64) // (num_v // n_cut + 1) + cols[r_edges].to(torch.int64) * n_cut
    else:
        block = cols[r_edges].to(torch.int64)
    return torch.bincount(block, minlength=num_v * n_cut).to(torch.int32)


def preprocess_direct(graph, n_cut):
    """truss_undirect_cuda2.py:118-141: returns the (tiled) out-list offsets,
    r_edges (edge ids stably sorted by head) and their (tiled) offsets re_ptr,
    all int32."""
    from .graph import tiling_row_ptr
    num_v = graph.num_vertices
    row_ptr = tiling_row_ptr(graph, n_cut) if n_cut > 1 else graph.row_ptr.to(torch.int32)
    r_edges = torch.argsort(graph.columns, stable=True).to(torch.int32)
    size_r = _in_list_sizes(graph.rows, graph.columns, r_edges, num_v, n_cut)
    re_ptr = torch.cat([torch.zeros(1, dtype=torch.int32, device=size_r.device), size_r.cumsum(0, dtype=torch.int32)])
    return row_ptr, r_edges, re_ptr


def preprocess_undirect(graph, n_cut_s, n_cut):
    """truss_undirect_cuda.py:80-121: returns (directed_ptr, columns_g,
    edges_id_nbr, row_ptr_g).  directed_ptr: the out-list offsets tiled by
    n_cut_s for the support count; slot v*n_cut+k of the symmetric adjacency
    lists the in-neighbours of v in tile k, then its out-neighbours in tile k."""
    from .graph import tiling_row_ptr
    num_v = graph.num_vertices
    dev = graph.columns.device
    directed_ptr = tiling_row_ptr(graph, n_cut_s) if n_cut_s > 1 else graph.row_ptr.to(torch.int32)
    r_edge = torch.argsort(graph.columns, stable=True).to(torch.int32)
    size_r = _in_list_sizes(graph.rows, graph.columns, r_edge, num_v, n_cut)
    out_ptr = tiling_row_ptr(graph, n_cut) if n_cut > 1 else graph.row_ptr.to(torch.int32)
    ptr_g = out_ptr.to(torch.int64).clone()
    ptr_g[1:] += size_r.cumsum(0)
    E = graph.columns.shape[0]
    columns_g = torch.zeros(2 * E, dtype=torch.int32, device=dev)
    edges_id_nbr = torch.zeros(2 * E, dtype=torch.int32, device=dev)
    out_idx = _batched_csr_selection(ptr_g[:-1] + size_r, ptr_g[1:])
    edges_id_nbr[out_idx] = torch.arange(E, dtype=torch.int32, device=dev)
    columns_g[out_idx] = graph.columns
    in_idx = _batched_csr_selection(ptr_g[:-1], ptr_g[:-1] + size_r)
    edges_id_nbr[in_idx] = r_edge
    columns_g[in_idx] = graph.rows[r_edge.to(torch.int64)]
    return directed_ptr, columns_g, edges_id_nbr, ptr_g.to(torch.int32)


def _e_map(keep):
    m = torch.zeros(keep.shape[0] + 1, dtype=torch.int32, device=keep.device)
    m[1:] = torch.cumsum(keep.int(), 0, dtype=torch.int32)
    return m


def _undirected_peel(support, edges, num_edges, peel, compact, compact_threshold):
    dev = support.device
    e_truss = []
    ptr_truss = [0]
    l = 1
    if support.shape[0] == 0:  # the reference's level search never ends here
        return 2, torch.zeros(0, dtype=torch.int32, device=dev), torch.zeros(1, dtype=torch.int32, device=dev)

    def next_level(support, l):
        in_curr = support == l
        while not bool(in_curr.any()):
            ptr_truss.append(ptr_truss[-1])
            l += 1
            in_curr = support == l
        return l, in_curr

    def done(l):
        e = torch.cat(e_truss) if e_truss else torch.zeros(0, dtype=torch.int32, device=dev)
        return l + 2, e, torch.tensor(ptr_truss, dtype=torch.int32, device=dev)

    l, in_curr = next_level(support, l)
    e_curr = torch.where(in_curr)[0].to(torch.int32)
    e_mask = torch.ones(support.shape[0], dtype=torch.bool, device=dev)
    count, n_out = 0, 0
    while True:
        while e_curr.shape[0] != 0:
            e_truss.append(edges[e_curr.long()])
            n_out += e_curr.shape[0]
            n_mark = torch.zeros(support.shape[0], dtype=torch.bool, device=dev)
            peel(e_curr, support, e_mask, n_mark, in_curr, l)
            e_mask[e_curr.long()] = False
            count += e_curr.shape[0]
            in_curr = n_mark
            e_curr = torch.where(n_mark)[0].to(torch.int32)
            if count + e_curr.shape[0] == num_edges():
                e_truss.append(edges[e_curr.long()])
                ptr_truss.append(n_out + e_curr.shape[0])
                return done(l)
        if count > compact_threshold:
            support, edges = compact(e_mask, support, edges)
            count = 0
            e_mask = torch.ones(support.shape[0], dtype=torch.bool, device=dev)
        ptr_truss.append(n_out)
        l, in_curr = next_level(support, l + 1)
        e_curr = torch.where(in_curr)[0].to(torch.int32)


def undirected_truss_direct(graph, row_ptr, r_edges, re_ptr, n_cut, compact_threshold=10000000):
    """truss_undirect_cuda2.py:145-280 (undirected_truss) with the oriented
    peel updates: returns (kmax, e_truss, ptr_truss).  row_ptr, r_edges, re_ptr
    come from preprocess_direct(graph, n_cut)."""
    g = {"rows": graph.rows, "cols": graph.columns, "rp": row_ptr, "r": r_edges, "re": re_ptr}
    support = support_computing(g["rows"], g["cols"], g["rp"], n_cut)

    def compact(keep, support, edges):
        g["cols"], g["rows"] = g["cols"][keep], g["rows"][keep]
        g["rp"] = update_row_ptr(keep, g["rp"])
        e_map = _e_map(keep)
        keep_r = keep[g["r"].long()]
        g["r"] = e_map[g["r"][keep_r].long()]
        g["re"] = update_row_ptr(keep_r, g["re"])
        return support[keep], edges[keep]

    edges = torch.arange(support.shape[0], dtype=torch.int32, device=support.device)
    support, edges = compact(support.bool(), support, edges)
    tile = n_cut > 1

    def peel(e_curr, support, e_mask, n_mark, in_curr, l):
        a = (e_curr, g["rows"], g["cols"])
        t = (support, e_mask, n_mark, in_curr, l)
        if tile:
            tt.peeling_direct_tile_oo(*a, g["rp"], *t, n_cut)
            tt.peeling_direct_tile_ii(*a, g["r"], g["re"], *t, n_cut)
            tt.peeling_direct_tile_oi(*a, g["rp"], g["r"], g["re"], *t, n_cut)
        else:
            tt.peeling_direct_oo(*a, g["rp"], *t)
            tt.peeling_direct_ii(*a, g["r"], g["re"], *t)
            tt.peeling_direct_oi(*a, g["rp"], g["r"], g["re"], *t)

    return _undirected_peel(support, edges, lambda: g["cols"].shape[0], peel, compact, compact_threshold)


def undirected_truss_undirect(graph, columns_g, edges_id_nbr, directed_ptr, row_ptr_g, n_cut_s, n_cut,
                              compact_threshold=10000000):
    """truss_undirect_cuda.py:125-235 (undirected_truss) with the symmetric
    peel update; inputs from preprocess_undirect(graph, n_cut_s, n_cut)."""
    g = {"rows": graph.rows, "cols": graph.columns, "cg": columns_g, "nbr": edges_id_nbr, "pg": row_ptr_g}
    support = support_computing(g["rows"], g["cols"], directed_ptr, n_cut_s)

    def compact(keep, support, edges):
        g["cols"], g["rows"] = g["cols"][keep], g["rows"][keep]
        e_map = _e_map(keep)
        keep_g = keep[g["nbr"].long()]
        g["cg"] = g["cg"][keep_g]
        g["nbr"] = e_map[g["nbr"][keep_g].long()]
        g["pg"] = update_row_ptr(keep_g, g["pg"])
        return support[keep], edges[keep]

    edges = torch.arange(support.shape[0], dtype=torch.int32, device=support.device)
    support, edges = compact(support.bool(), support, edges)

    def peel(e_curr, support, e_mask, n_mark, in_curr, l):
        if n_cut > 1:
            tt.peeling_undirect_tile(e_curr, g["rows"], g["cols"], g["cg"], g["pg"], g["nbr"], support, e_mask,
                                     n_mark, in_curr, l, n_cut)
        else:
            tt.peeling_undirect(e_curr, g["rows"], g["cols"], g["cg"], g["pg"], g["nbr"], support, e_mask, n_mark,
                                in_curr, l)

    return _undirected_peel(support, edges, lambda: g["cols"].shape[0], peel, compact, compact_threshold)


# ------------------------------------------------------------------ tensor_original driver
def symmetric_csr(graph):
    """Both directions of every edge of `graph` (rows sorted by column): the
    CSRGraph the tensor_original driver reads.  Returns (row_ptr int32,
    columns int32)."""
    V = graph.num_vertices
    r = torch.cat([graph.rows, graph.columns]).to(torch.int64)
    c = torch.cat([graph.columns, graph.rows]).to(torch.int64)
    key = r * (V + 1) + c
    order = torch.argsort(key)
    r, c = r[order], c[order]
    rp = torch.zeros(V + 1, dtype=torch.int32, device=c.device)
    rp[1:] = torch.cumsum(torch.bincount(r, minlength=V), 0).to(torch.int32)
    return rp, c.to(torch.int32)


def _selection_opt2(starts, ends):
    """batched_csr_selection_opt2 (helper.py:102-121) on non-empty ranges."""
    return _csr_selection_ptr(starts, ends)


def truss_tensor_original(row_ptr, columns, compact_threshold=100000):
    """demo_truss/tensor_original/truss_nosavetri_tensor4.py:27-196
    (truss_deposs) over a symmetric CSR (row_ptr, columns int32 on the GPU),
    written against segment_isin2, segment_isinis_m and sub_suppport_affect:
    returns (e_truss, ptr_truss) over the undirected edges u < v in CSR order.
    As in the reference, the edges of the last sub-round are not appended to
    e_truss (the loop stops first, :147-152)."""
    dev = columns.device
    V = row_ptr.shape[0] - 1
    row_ptr = row_ptr.to(torch.int64)
    columns = columns.to(torch.int32)
    row_indice_g = torch.repeat_interleave(torch.arange(V, dtype=torch.int32, device=dev), row_ptr[1:] - row_ptr[:-1])
    mask = row_indice_g < columns
    row_indice = row_indice_g[mask]
    cols_u = columns[mask]
    Eu = cols_u.shape[0]
    e_truss, ptr_truss = [], [0]
    e_mask = torch.ones(Eu, dtype=torch.bool, device=dev)
    edges_id = torch.arange(Eu, dtype=torch.int32, device=dev)
    edges_id_nbr = torch.arange(columns.shape[0], dtype=torch.int32, device=dev)
    edges_id_nbr[mask] = edges_id
    sorted_indices = torch.argsort(columns[~mask], stable=True)
    temp = torch.zeros(Eu, dtype=torch.int32, device=dev)
    temp[sorted_indices] = edges_id
    edges_id_nbr[~mask] = temp
    rp32 = row_ptr.to(torch.int32)
    direc = torch.zeros(V, dtype=torch.int32, device=dev)
    tt.segment_add(mask.int(), rp32, direc)
    direc_rp = torch.cat([torch.zeros(1, dtype=torch.int32, device=dev), direc.cumsum(0, dtype=torch.int32)])
    support = torch.zeros(Eu, dtype=torch.int32, device=dev)
    tt.segment_isin2(row_indice, cols_u, direc_rp, support)
    e_mask[edges_id[support == 0].long()] = False
    if not bool(e_mask.any()):
        return torch.zeros(0, dtype=torch.int32, device=dev), torch.tensor(ptr_truss, dtype=torch.int32)
    keep = e_mask[edges_id_nbr.long()]
    edges_id_nbr = edges_id_nbr[keep]
    columns = columns[keep]
    row_ptr = update_row_ptr(keep, rp32).to(torch.int64)
    n_out = [0]

    def level_edges(l):
        return torch.where(support == l)[0].to(torch.int32)

    l = 1
    e_curr = level_edges(l)
    while e_curr.shape[0] == 0:
        ptr_truss.append(n_out[0])
        l += 1
        e_curr = level_edges(l)
    e_del = 0
    columns = torch.cat([columns, torch.full((1,), -1, dtype=torch.int32, device=dev)])
    while True:
        e_truss.append(edges_id[e_curr.long()])
        n_out[0] += e_curr.shape[0]
        ec = e_curr.long()
        left, s_ptr = _selection_opt2(row_ptr[row_indice[ec].long()], row_ptr[row_indice[ec].long() + 1])
        right, e_ptr = _selection_opt2(row_ptr[cols_u[ec].long()], row_ptr[cols_u[ec].long() + 1])
        m1 = e_mask[edges_id_nbr[left].long()]
        m2 = e_mask[edges_id_nbr[right].long()]
        left = left.clone()
        right = right.clone()
        left[~m1] = -1
        right[~m2] = -1
        mk1 = torch.zeros(left.shape[0], dtype=torch.bool, device=dev)
        mk2 = torch.zeros(right.shape[0], dtype=torch.bool, device=dev)
        tt.segment_isinis_m(columns[left], s_ptr, columns[right], e_ptr, mk1, mk2)
        left_nbr = edges_id_nbr[left[mk1]]
        right_nbr = edges_id_nbr[right[mk2]]
        if left_nbr.shape[0] == 0 or right_nbr.shape[0] == 0:
            e_mask[ec] = False
            e_curr = left_nbr
        else:
            values = torch.zeros(e_ptr.shape[0] - 1, dtype=torch.int32, device=dev)
            tt.segment_add(mk2.int(), e_ptr, values)
            e_curr_rep = torch.repeat_interleave(e_curr, values.long())
            s1 = support[left_nbr.long()] > l
            s2 = support[right_nbr.long()] > l
            affect = torch.zeros(e_mask.shape[0], dtype=torch.bool, device=dev)
            tt.sub_suppport_affect(left_nbr, right_nbr, e_curr_rep, support, s1, s2, affect, l)
            e_del += e_curr.shape[0]
            e_mask[ec] = False
            e_aff = torch.where(affect)[0]
            e_curr = e_aff[support[e_aff] <= l].to(torch.int32)
        if int(e_mask.sum()) == e_curr.shape[0]:
            ptr_truss.append(n_out[0])
            break
        if e_del >= compact_threshold:
            keep = e_mask[edges_id_nbr.long()]
            edges_id_nbr = edges_id_nbr[keep]
            columns = torch.cat([columns[:-1][keep], torch.full((1,), -1, dtype=torch.int32, device=dev)])
            row_ptr = update_row_ptr(keep, row_ptr.to(torch.int32)).to(torch.int64)
            e_del = 0
            idx = torch.where(e_mask)[0]
            edges_id, support, cols_u, row_indice = edges_id[idx], support[idx], cols_u[idx], row_indice[idx]
            remap = torch.zeros(e_mask.shape[0], dtype=torch.int32, device=dev)
            remap[idx] = torch.arange(idx.shape[0], dtype=torch.int32, device=dev)
            e_curr = remap[e_curr.long()]
            edges_id_nbr = remap[edges_id_nbr.long()]
            e_mask = torch.ones(idx.shape[0], dtype=torch.bool, device=dev)
        if e_curr.shape[0] == 0:
            ptr_truss.append(n_out[0])
            l += 1
            e_curr = level_edges(l)
            while e_curr.shape[0] == 0:
                ptr_truss.append(n_out[0])
                l += 1
                e_curr = level_edges(l)
    e = torch.cat(e_truss) if e_truss else torch.zeros(0, dtype=torch.int32, device=dev)
    return e, torch.tensor(ptr_truss, dtype=torch.int32)
