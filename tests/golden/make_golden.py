"""Generate the golden fixtures from the reference's OWN code (run in a
container that has the reference tree; the fixtures are committed and the
tests never read the reference tree).

For each case graph (an edge list) this records:
  * the reference preprocessing (src/type/CSRCOO.py read_graph -> CSRCOO:
    rows, columns, row_ptr, and the rank -> original-id vertex list);
  * the support from the reference's own OpenMP operator
    (myhpu_extension_opmp.cpp segment_isin2tile_cpu, built into oracle/_ref);
  * e_truss / ptr_truss / kmax of the reference driver
    singlegpu_truss.k_truss (the `--cuda` flow) for n_cut = 1 and 2.  Its
    sub_AllAffectedSupport_(tile)not op has no CPU twin in the reference, so
    here it runs the oracle's restatement; every other op is the reference's;
  * e_truss / ptr_truss of demo_truss/test/truss_setup.k_truss (the
    reference's CPU path: all of its ops are the reference's own OpenMP code);
  * the k-truss edge sets of ktruss_search/ktruss_cuda.k_truss (its pycuda
    kernels replaced by the oracle restatement, its segment_add/isin kernels
    by the reference's OpenMP operators) for several k;
  * networkx truss numbers (independent check).
The reference drivers return only kmax (singlegpu_truss.py:158), so e_truss
and ptr_truss are read from the function's frame at return (sys.setprofile).

Usage: python tests/golden/make_golden.py   (writes tests/golden/*.npz)
"""
import contextlib
import io
import os
import sys
import tempfile
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("TDT_REFERENCE_ROOT", "/root/reference")
sys.path.insert(0, REPO)
sys.dont_write_bytecode = True

from oracle import oracle as O  # noqa: E402
from tdtdecomposition_gb300 import generators as G  # noqa: E402


# ---------------------------------------------------------------- shims
def _np(t):
    a = t.numpy()
    return a.view(np.uint8) if a.dtype == np.bool_ else a


def _install_shims():
    R = O.ref_ops()
    if R is None:
        raise SystemExit("oracle/_ref could not be built (reference tree missing?)")

    def segment_add(col_indices, col_ptr, output):
        R.ref_segment_add(_np(col_indices), _np(col_ptr), _np(output), output.shape[0])

    def segment_isin2(a_rows, cols, rp, output):
        R.ref_segment_isin2(_np(a_rows), _np(cols), _np(rp), _np(output), output.shape[0])

    def segment_isin2tile(a_rows, cols, rp, n_cut, output):
        R.ref_segment_isin2tile(_np(a_rows), _np(cols), _np(rp), int(n_cut), _np(output),
                                output.shape[0] * int(n_cut))

    def sub_AllAffectedSupport(e_affect, a_rows, cols, rp, mark, l, n_mark, output):
        R.ref_all_affected_support(_np(e_affect), _np(a_rows), _np(cols), _np(rp), _np(mark), int(l),
                                   _np(n_mark), _np(output), e_affect.shape[0])

    def sub_AllAffectedSupport_tile(e_affect, a_rows, cols, rp, n_cut, mark, l, n_mark, output):
        R.ref_all_affected_support_tile(_np(e_affect), _np(a_rows), _np(cols), _np(rp), int(n_cut), _np(mark),
                                        int(l), _np(n_mark), _np(output), e_affect.shape[0] * int(n_cut))

    def sub_AllAffectedSupport_not(e_affect, a_rows, cols, rp, mark, l, n_mark, output):
        O.all_affected_support_tilenot(_np(e_affect), _np(a_rows), _np(cols), _np(rp), 1, _np(mark), l,
                                       _np(n_mark), _np(output))

    def sub_AllAffectedSupport_tilenot(e_affect, a_rows, cols, rp, n_cut, mark, l, n_mark, output):
        O.all_affected_support_tilenot(_np(e_affect), _np(a_rows), _np(cols), _np(rp), n_cut, _np(mark), l,
                                       _np(n_mark), _np(output))

    tt = types.ModuleType("trusstensor")
    for f in (segment_add, segment_isin2, segment_isin2tile, sub_AllAffectedSupport, sub_AllAffectedSupport_tile,
              sub_AllAffectedSupport_not, sub_AllAffectedSupport_tilenot):
        setattr(tt, f.__name__, f)
    sys.modules["trusstensor"] = tt
    mc = types.ModuleType("mycudaf")
    for f in (segment_isin2tile, sub_AllAffectedSupport, sub_AllAffectedSupport_tile):
        setattr(mc, f.__name__, f)
    sys.modules["mycudaf"] = mc

    # pycuda: SourceModule kernels of ktruss_cuda.py run as CPU restatements
    def _arg(a):
        return _np(a.t) if hasattr(a, "t") else a

    kernels = {
        "segmentAddKernel": lambda c, p, o, n: R.ref_segment_add(_arg(c), _arg(p), _arg(o), int(n)),
        "checkElementsTwoPtr": lambda r, c, p, o, n: R.ref_segment_isin2(_arg(r), _arg(c), _arg(p), _arg(o), int(n)),
        "checkElementsTwoPtrTile": lambda r, c, p, nc, o, n: R.ref_segment_isin2tile(
            _arg(r), _arg(c), _arg(p), int(nc), _arg(o), int(n)),
        "checkElementsTwoPtr_k": lambda r, c, p, k, o, n: O.lib().orc_segment_isin2tile_k(
            _arg(r), _arg(c), _arg(p), 1, int(k), _arg(o), int(n)),
        "checkElementsTwoPtrTile_k": lambda r, c, p, nc, k, o, n: O.lib().orc_segment_isin2tile_k(
            _arg(r), _arg(c), _arg(p), int(nc), int(k), _arg(o), int(n) // int(nc)),
        "subAffectedSupport": lambda r, c, p, m, o, n: O.lib().orc_sub_affected_support_tile(
            _arg(r), _arg(c), _arg(p), 1, _arg(m), _arg(o), int(n)),
        "subAffectedSupport_tile": lambda r, c, p, nc, m, o, n: O.lib().orc_sub_affected_support_tile(
            _arg(r), _arg(c), _arg(p), int(nc), _arg(m), _arg(o), int(n) // int(nc)),
    }

    class _Mod:
        def __init__(self, code):
            pass

        def get_function(self, name):
            f = kernels[name]
            return lambda *args, block=None, grid=None: f(*args)

    class PointerHolderBase:
        def __init__(self):
            pass

    pc = types.ModuleType("pycuda")
    pc.autoinit = types.ModuleType("pycuda.autoinit")
    pc.compiler = types.ModuleType("pycuda.compiler")
    pc.compiler.SourceModule = _Mod
    pc.driver = types.ModuleType("pycuda.driver")
    pc.driver.PointerHolderBase = PointerHolderBase
    for name, mod in (("pycuda", pc), ("pycuda.autoinit", pc.autoinit), ("pycuda.compiler", pc.compiler),
                      ("pycuda.driver", pc.driver)):
        sys.modules[name] = mod
    torch.cuda.synchronize = lambda *a, **k: None


def _import_ref(modname, relpath):
    import importlib.util
    for p in (REF, os.path.join(REF, "demo_truss")):
        if p not in sys.path:
            sys.path.insert(0, p)
    spec = importlib.util.spec_from_file_location(modname, os.path.join(REF, relpath))
    mod = importlib.util.module_from_spec(spec)
    with contextlib.redirect_stdout(io.StringIO()):
        spec.loader.exec_module(mod)
    return mod


def _capture_locals(fn, names, *args):
    """Call fn(*args) and return (its result, {name: local at return})."""
    got = {}
    code = fn.__code__

    def prof(frame, event, arg):
        if event == "return" and frame.f_code is code:
            for n in names:
                if n in frame.f_locals:
                    got[n] = frame.f_locals[n]

    old = sys.getprofile()
    sys.setprofile(prof)
    try:
        with contextlib.redirect_stdout(io.StringIO()):
            res = fn(*args)
    finally:
        sys.setprofile(old)
    return res, got


# ---------------------------------------------------------------- cases
def _cases():
    import networkx as nx
    cases = {}
    cases["fixture"] = np.loadtxt(os.path.join(REF, "test_data/example_graph.txt"), dtype=np.int32)
    s, d = G.er_edges(512, 4096, seed=0)
    cases["er_512_4096"] = np.stack([s, d], 1)
    s, d = G.ba_edges(1500, 8, seed=1000)
    cases["ba_1500_8"] = np.stack([s, d], 1)
    s, d = G.rmat_edges(10, 16 * 1024, seed=1)
    cases["rmat_s10"] = np.stack([s, d], 1)
    g = nx.powerlaw_cluster_graph(1500, 6, 0.6, seed=3)
    cases["plc_1500"] = np.array(list(g.edges()), dtype=np.int32)
    # cliques of sizes 5..9 chained by paths, ids shuffled: deep levels, empty levels
    rng = np.random.default_rng(5)
    edges, base = [], 0
    for k in (5, 6, 7, 9):
        for a in range(k):
            for b in range(a + 1, k):
                edges.append((base + a, base + b))
        edges.append((base + k - 1, base + k))
        base += k + 1
    perm = rng.permutation(base + 1)
    cases["cliques"] = perm[np.array(edges, dtype=np.int64)].astype(np.int32)
    s, d = G.er_edges(4096, 65536, seed=0)
    cases["er_4096_65536"] = np.stack([s, d], 1)
    return cases


def _nx_truss(pairs):
    import networkx as nx
    g = nx.Graph()
    g.add_edges_from(pairs.tolist())
    g.remove_edges_from(nx.selfloop_edges(g))
    out = {}
    k = 2
    h = g
    while h.number_of_edges():
        h = nx.k_truss(h, k)
        for u, v in h.edges():
            out[(min(u, v), max(u, v))] = k
        k += 1
    return out


def main():
    _install_shims()
    sys.path.insert(0, REF)
    from src.type.CSRCOO import CSRCOO  # the reference's own module
    sg = _import_ref("singlegpu_truss", "demo_truss/singlegpu_truss.py")
    ts = _import_ref("truss_setup", "demo_truss/test/truss_setup.py")
    kt = _import_ref("ktruss_cuda", "demo_truss/ktruss_search/ktruss_cuda.py")
    R = O.ref_ops()
    for name, pairs in _cases().items():
        out = {"pairs": pairs.astype(np.int32)} if name != "er_4096_65536" else {}
        with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
            np.savetxt(f, pairs, fmt="%d")
            path = f.name
        with contextlib.redirect_stdout(io.StringIO()):
            graph, v2i = CSRCOO.read_graph(path, directed=True)
        os.unlink(path)
        rows = graph.rows.numpy().astype(np.int32)
        cols = graph.columns.numpy().astype(np.int32)
        rp = graph.row_ptr.numpy().astype(np.int32)
        V = rp.shape[0] - 1
        verts = np.zeros(V, np.int64)
        for vid, idx in v2i.items():
            verts[idx] = vid
        out.update(ref_rows=rows, ref_cols=cols, ref_rp=rp, ref_vertices=verts)
        # reference support (its own OpenMP op), untiled
        sup = np.zeros(cols.shape[0], np.int32)
        R.ref_segment_isin2(rows, cols, rp, sup, cols.shape[0])
        out["ref_support"] = sup
        for n_cut in (1, 2):
            g2 = CSRCOO(columns=torch.from_numpy(cols.copy()), row_ptr=torch.from_numpy(rp.copy()),
                        rows=torch.from_numpy(rows.copy()))
            if n_cut > 1:
                with contextlib.redirect_stdout(io.StringIO()):
                    sg.csr_to_tilingcsr(g2, V // n_cut, n_cut)
            out["ref_rp_tiled%d" % n_cut] = g2.row_ptr.numpy().astype(np.int32).copy()
            sup_t = np.zeros(cols.shape[0], np.int32)
            R.ref_segment_isin2tile(rows, cols, out["ref_rp_tiled%d" % n_cut], n_cut, sup_t, cols.shape[0] * n_cut)
            assert np.array_equal(sup_t, sup), name
            res, loc = _capture_locals(sg.k_truss, ("e_truss", "ptr_truss"), g2, n_cut, V)
            out["sg_kmax%d" % n_cut] = np.int64(res[0])
            out["sg_e_truss%d" % n_cut] = loc["e_truss"].numpy().astype(np.int32)
            out["sg_ptr_truss%d" % n_cut] = loc["ptr_truss"].numpy().astype(np.int32)
        g3 = CSRCOO(columns=torch.from_numpy(cols.copy()), row_ptr=torch.from_numpy(out["ref_rp_tiled2"].copy()),
                    rows=torch.from_numpy(rows.copy()))
        res, loc = _capture_locals(ts.k_truss, ("e_truss", "ptr_truss"), g3, 2, V)
        out["cpu_kmax"] = np.int64(res[0])
        out["cpu_e_truss"] = loc["e_truss"].numpy().astype(np.int32)
        out["cpu_ptr_truss"] = loc["ptr_truss"].numpy().astype(np.int32)
        kmax = int(out["sg_kmax2"])
        ks = sorted({3, 4, 5, max(3, kmax // 2), kmax, kmax + 1})
        out["kt_ks"] = np.array(ks, np.int32)
        for k in ks:
            g4 = CSRCOO(columns=torch.from_numpy(cols.copy()), row_ptr=torch.from_numpy(out["ref_rp_tiled2"].copy()),
                        rows=torch.from_numpy(rows.copy()))
            (e_rest, _, _), _ = _capture_locals(kt.k_truss, (), g4, k - 2, 2, V)
            er = e_rest.numpy()
            out["kt_rows_k%d" % k] = g4.rows.numpy()[er].astype(np.int32)
            out["kt_cols_k%d" % k] = g4.columns.numpy()[er].astype(np.int32)
        if name != "er_4096_65536":
            nt = _nx_truss(pairs)
            keys = np.array(sorted(nt), np.int64).reshape(-1, 2)
            out["nx_pairs"] = keys.astype(np.int32)
            out["nx_truss"] = np.array([nt[tuple(k)] for k in keys], np.int32)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("%-16s V=%6d E=%7d kmax=%d" % (name, V, cols.shape[0], kmax), flush=True)
    # demo_truss/test/truss_setup.py:263-266 also holds a hand-made tiled CSR,
    # but its column 4 has no row_ptr entry (4 vertices of row_ptr, 5 ids), so
    # the reference operator reads past row_ptr on it; it is not a usable
    # golden vector.


if __name__ == "__main__":
    main()
