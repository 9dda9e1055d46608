"""On-disk graph formats of the reference, read and written here.

* Text edge lists (`Graph.read_edgelist`, src/type/Graph_Truss.py:177-213):
  whitespace-separated integer pairs, one edge per line; lines starting with
  '#' or '%' are skipped.  :func:`read_graph` is `CSRCOO.read_graph`
  (src/type/CSRCOO.py:165-167) with the dedup / degree rank / CSR build done
  on the GPU (:func:`preprocess.preprocess_edges`).
* `.pth` files of `read_prepro_save` (demo_truss/singlegpu_truss.py:172-178):
  `torch.save` of the reference's `src.type.CSRCOO.CSRCOO` object (attributes
  rows, columns, row_ptr, plus the `Graph` base's directed, vertices_t,
  edges_t).  :func:`load_pth` reads those files (and this package's own
  tensor-only format) with an unpickler that resolves only torch and that
  class; :func:`save_pth` writes either format, the reference one loadable by
  the reference's `torch.load(args.output)` (:183).
* Binary CSR of demo_truss/test/txt_to_csrcoo.cpp:56-104: `csr_vlist.bin`
  (int64[V+1] offsets) and `csr_elist.bin` (int32 neighbours) of the
  symmetric graph, vertex ids renumbered in increasing order, self-loops and
  duplicates removed.  :func:`read_csr_bin` / :func:`write_csr_bin`.
"""
import os
import pickle
import sys
import types

import numpy as np
import torch

from .graph import CSRCOO

_OWN_FORMAT = "tdtdecomposition_gb300.csrcoo.v1"
_REF_MODULE, _REF_CLASS = "src.type.CSRCOO", "CSRCOO"


# ---------------------------------------------------------------- text edge lists
def read_edgelist(path):
    """(src, dst) int32 arrays of the edge list in `path` (self-loops and
    duplicates are kept; preprocessing removes them)."""
    with open(path, "rb") as f:
        data = f.read()
    lines = [l for l in data.splitlines() if l.strip() and l.lstrip()[:1] not in (b"#", b"%")]
    if not lines:
        return np.zeros(0, np.int32), np.zeros(0, np.int32)
    arr = np.array([l.split()[:2] for l in lines], dtype=np.int64)
    if arr.min() < 0 or arr.max() > np.iinfo(np.int32).max:
        raise ValueError("vertex ids must lie in [0, 2^31)")
    return arr[:, 0].astype(np.int32), arr[:, 1].astype(np.int32)


def read_graph(path, device="cuda", workspace=None):
    """Text edge list -> (degree-oriented CSRCOO on `device`, vertices: the
    original id of every rank), as CSRCOO.read_graph; the preprocessing runs
    on the GPU."""
    from .preprocess import preprocess_edges
    s, d = read_edgelist(path)
    dev = torch.device(device)
    return preprocess_edges(torch.as_tensor(s).to(dev), torch.as_tensor(d).to(dev), workspace=workspace)


# ---------------------------------------------------------------- .pth
class _RefCSRCOO:
    """Stand-in for src.type.CSRCOO.CSRCOO while unpickling."""

    def __setstate__(self, state):
        self.__dict__.update(state)


class _Unpickler(pickle.Unpickler):
    """Resolves torch's own reconstruction helpers, OrderedDict, and the
    reference's CSRCOO class; refuses everything else."""

    def find_class(self, module, name):
        if module == _REF_MODULE and name == _REF_CLASS:
            return _RefCSRCOO
        if module == "collections" and name == "OrderedDict":
            return super().find_class(module, name)
        if module == "torch" or module.startswith("torch."):
            return super().find_class(module, name)
        raise pickle.UnpicklingError("refusing to load %s.%s from a graph file" % (module, name))


_pickle_module = types.ModuleType("tdt_graph_pickle")
_pickle_module.Unpickler = _Unpickler
_pickle_module.load = pickle.load
_pickle_module.loads = pickle.loads
_pickle_module.__name__ = "tdt_graph_pickle"


def load_pth(path, map_location="cpu"):
    """CSRCOO from a `.pth` written by the reference's read_prepro_save or by
    :func:`save_pth`."""
    obj = torch.load(path, map_location=map_location, weights_only=False, pickle_module=_pickle_module)
    if isinstance(obj, dict) and obj.get("format") == _OWN_FORMAT:
        return CSRCOO(columns=obj["columns"], row_ptr=obj["row_ptr"], rows=obj["rows"])
    if isinstance(obj, _RefCSRCOO):
        st = obj.__dict__
        return CSRCOO(columns=st["columns"], row_ptr=st["row_ptr"], rows=st["rows"])
    raise ValueError("%s holds neither a reference CSRCOO nor a %s graph" % (path, _OWN_FORMAT))


def save_pth(graph, path, reference_compatible=True):
    """Write `graph` (host copies of its tensors).  reference_compatible: as the
    reference's own `src.type.CSRCOO.CSRCOO` object, which its drivers load
    with torch.load; otherwise a plain dict of tensors."""
    t = {"rows": graph.rows.detach().cpu(), "columns": graph.columns.detach().cpu(),
         "row_ptr": graph.row_ptr.detach().cpu()}
    if not reference_compatible:
        torch.save(dict(t, format=_OWN_FORMAT), path)
        return
    # pickle names the class by module path: give it one, borrowing the real
    # class when the reference's package is importable
    stubs = {}
    mod = sys.modules.get(_REF_MODULE)
    cls = getattr(mod, _REF_CLASS, None) if mod is not None else None
    if cls is None:
        cls = type(_REF_CLASS, (), {"__module__": _REF_MODULE})
        for name in ("src", "src.type", _REF_MODULE):
            if name not in sys.modules:
                stubs[name] = types.ModuleType(name)
                sys.modules[name] = stubs[name]
        setattr(sys.modules[_REF_MODULE], _REF_CLASS, cls)
    try:
        obj = cls.__new__(cls)
        obj.__dict__.update({"directed": True, "vertices_t": None, "edges_t": None}, **t)
        torch.save(obj, path)
    finally:
        for name in stubs:
            sys.modules.pop(name, None)


# ---------------------------------------------------------------- binary CSR
def write_csr_bin(out_dir, src, dst):
    """Write the symmetric CSR of edge list (src, dst) as txt_to_csrcoo does:
    drop self-loops, renumber the vertex ids in increasing order, both
    directions of every edge, sorted, duplicates removed."""
    s = np.asarray(src, np.int64)
    d = np.asarray(dst, np.int64)
    keep = s != d
    s, d = s[keep], d[keep]
    ids = np.unique(np.concatenate([s, d]))
    a = np.searchsorted(ids, np.concatenate([s, d]))
    b = np.searchsorted(ids, np.concatenate([d, s]))
    key = np.unique(a * len(ids) + b) if len(ids) else np.zeros(0, np.int64)
    a, b = key // max(len(ids), 1), key % max(len(ids), 1)
    vlist = np.zeros(len(ids) + 1, np.int64)
    np.add.at(vlist, a + 1, 1)
    vlist = np.cumsum(vlist).astype(np.int64)
    os.makedirs(out_dir, exist_ok=True)
    vlist.tofile(os.path.join(out_dir, "csr_vlist.bin"))
    b.astype(np.int32).tofile(os.path.join(out_dir, "csr_elist.bin"))
    return ids


def read_csr_bin(in_dir):
    """(src, dst) int32 with src < dst, one per undirected edge, from the
    csr_vlist.bin / csr_elist.bin pair in `in_dir`."""
    vlist = np.fromfile(os.path.join(in_dir, "csr_vlist.bin"), dtype=np.int64)
    elist = np.fromfile(os.path.join(in_dir, "csr_elist.bin"), dtype=np.int32)
    if len(vlist) == 0 or vlist[0] != 0 or vlist[-1] != len(elist) or np.any(np.diff(vlist) < 0):
        raise ValueError("csr_vlist.bin / csr_elist.bin do not form a CSR")
    u = np.repeat(np.arange(len(vlist) - 1, dtype=np.int64), np.diff(vlist))
    m = u < elist
    return u[m].astype(np.int32), elist[m].astype(np.int32)
