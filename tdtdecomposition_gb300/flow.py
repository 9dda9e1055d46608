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


def k_truss(graph, n_cut, num_v, cpu_flow=False, compact_threshold=1000000):
    """singlegpu_truss.py:67-158 (cpu_flow=False, peel update = *_not) or
    test/truss_setup.py:61-154 (cpu_flow=True, peel update = sub_AllAffectedSupport*).
    Mutates graph like the reference.  Returns (kmax, e_truss, ptr_truss)."""
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
        else:
            all_affect_support_not(e_affect, graph, n_cut, e_mask, l, n_mark, support)
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
