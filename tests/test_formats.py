"""On-disk formats (formats.py): text edge lists, the reference's `.pth`
CSRCOO pickles, and the binary CSR of txt_to_csrcoo.cpp."""
import os
import pickle
import shutil
import subprocess
import sys

import numpy as np
import pytest
import torch

from tdtdecomposition_gb300 import formats as F
from tdtdecomposition_gb300.graph import CSRCOO
from tests import _golden as GD

# golden files written by the reference's own converter and CSRCOO class
# (tests/golden/make_format_golden.py); the reference tree itself is used only
# when TDT_REFERENCE_ROOT names it
REF = os.environ.get("TDT_REFERENCE_ROOT")
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _write_text(path, pairs, header=True):
    with open(path, "w") as f:
        if header:
            f.write("# an edge list\n% with two comment styles\n")
        for a, b in pairs:
            f.write("%d\t%d\n" % (a, b))


def _graph():
    d = GD.load("fixture")
    return CSRCOO(columns=torch.as_tensor(d["ref_cols"], dtype=torch.int32),
                  row_ptr=torch.as_tensor(d["ref_rp"], dtype=torch.int64),
                  rows=torch.as_tensor(d["ref_rows"], dtype=torch.int32))


def test_read_edgelist_skips_comments(tmp_path):
    pairs = GD.load("fixture")["pairs"]
    p = tmp_path / "g.txt"
    _write_text(p, pairs)
    s, d = F.read_edgelist(str(p))
    assert s.dtype == np.int32 and np.array_equal(np.stack([s, d], 1), pairs)


def test_read_edgelist_empty_and_bad_ids(tmp_path):
    p = tmp_path / "e.txt"
    p.write_text("# nothing\n")
    s, d = F.read_edgelist(str(p))
    assert len(s) == 0 and len(d) == 0
    p.write_text("1 -2\n")
    with pytest.raises(ValueError):
        F.read_edgelist(str(p))


@pytest.mark.parametrize("ref_compat", [True, False])
def test_pth_round_trip(tmp_path, ref_compat):
    g = _graph()
    p = str(tmp_path / "g.pth")
    F.save_pth(g, p, reference_compatible=ref_compat)
    h = F.load_pth(p)
    for a in ("rows", "columns", "row_ptr"):
        assert torch.equal(getattr(g, a), getattr(h, a))
    assert "src.type.CSRCOO" not in sys.modules


def test_pth_loader_refuses_other_classes(tmp_path):
    class Evil:
        def __reduce__(self):
            return (os.getcwd, ())
    p = str(tmp_path / "evil.pth")
    torch.save({"x": Evil()}, p)
    with pytest.raises(pickle.UnpicklingError):
        F.load_pth(p)


def test_pth_written_by_the_reference_class_loads_here():
    """A file torch.save wrote from the reference's own CSRCOO class (int32
    row_ptr, as read_prepro_save writes it) loads as the same graph."""
    g = _graph()
    h = F.load_pth(os.path.join(GOLDEN, "fmt_ref_csrcoo.pth"))
    assert torch.equal(h.columns, g.columns) and torch.equal(h.rows, g.rows)
    assert torch.equal(h.row_ptr.to(torch.int64), g.row_ptr)


@pytest.mark.skipif(REF is None or not os.path.isdir(os.path.join(REF, "src")),
                    reason="TDT_REFERENCE_ROOT does not name the reference tree")
def test_pth_interoperates_with_the_reference_class(tmp_path):
    """Our reference-compatible file loads as the reference's own CSRCOO, and a
    file the reference's class wrote loads here."""
    g = _graph()
    ours = str(tmp_path / "ours.pth")
    theirs = str(tmp_path / "theirs.pth")
    F.save_pth(g, ours)
    code = r"""
import sys, torch
sys.path.insert(0, %r)
from src.type.CSRCOO import CSRCOO
g = torch.load(%r, weights_only=False)
assert type(g) is CSRCOO, type(g)
assert g.num_vertices == %d and g.num_edges == %d
torch.save(CSRCOO(columns=g.columns, row_ptr=g.row_ptr.to(torch.int32), rows=g.rows), %r)
""" % (REF, ours, g.num_vertices, g.num_edges, theirs)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    h = F.load_pth(theirs)
    assert torch.equal(h.columns, g.columns) and torch.equal(h.rows, g.rows)
    assert torch.equal(h.row_ptr.to(torch.int64), g.row_ptr)


def test_binary_csr_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    s = rng.integers(0, 500, 3000).astype(np.int32) * 7
    d = rng.integers(0, 500, 3000).astype(np.int32) * 7
    ids = F.write_csr_bin(str(tmp_path), s, d)
    a, b = F.read_csr_bin(str(tmp_path))
    keep = s != d
    u = np.minimum(s[keep], d[keep])
    v = np.maximum(s[keep], d[keep])
    want = set(zip(np.searchsorted(ids, u).tolist(), np.searchsorted(ids, v).tolist()))
    assert set(zip(a.tolist(), b.tolist())) == want and len(a) == len(want)


def test_binary_csr_matches_reference_tool(tmp_path):
    """write_csr_bin produces the same bytes as the reference's converter
    (txt_to_csrcoo.cpp) wrote for the same edge list."""
    pairs = np.load(os.path.join(GOLDEN, "fmt_csr_pairs.npy"))
    F.write_csr_bin(str(tmp_path / "ours"), pairs[:, 0], pairs[:, 1])
    for name in ("csr_vlist.bin", "csr_elist.bin"):
        with open(os.path.join(GOLDEN, "fmt_csr_ref", name), "rb") as f:
            assert (tmp_path / "ours" / name).read_bytes() == f.read(), name


@pytest.mark.skipif(REF is None or not os.path.isfile(os.path.join(str(REF), "demo_truss/test/txt_to_csrcoo.cpp"))
                    or shutil.which("g++") is None, reason="TDT_REFERENCE_ROOT does not name the reference tree")
def test_binary_csr_matches_reference_tool_live(tmp_path):
    """The same against the reference's converter built and run here."""
    rng = np.random.default_rng(5)
    pairs = rng.integers(0, 300, size=(2000, 2)) * 3 + 1
    txt = tmp_path / "g.txt"
    _write_text(txt, pairs, header=False)
    exe = tmp_path / "txt_to_csrcoo"
    subprocess.run(["g++", "-O2", "-o", str(exe), os.path.join(REF, "demo_truss/test/txt_to_csrcoo.cpp")],
                   check=True, capture_output=True)
    (tmp_path / "ref").mkdir()
    subprocess.run([str(exe), str(txt), str(tmp_path / "ref")], check=True, capture_output=True)
    F.write_csr_bin(str(tmp_path / "ours"), pairs[:, 0], pairs[:, 1])
    for name in ("csr_vlist.bin", "csr_elist.bin"):
        assert (tmp_path / "ours" / name).read_bytes() == (tmp_path / "ref" / name).read_bytes(), name


def test_read_csr_bin_rejects_garbage(tmp_path):
    np.array([0, 5], np.int64).tofile(tmp_path / "csr_vlist.bin")
    np.array([1, 2], np.int32).tofile(tmp_path / "csr_elist.bin")
    with pytest.raises(ValueError):
        F.read_csr_bin(str(tmp_path))


@pytest.mark.gpu
def test_read_graph_on_gpu_decomposes_like_the_reference(tmp_path):
    from tdtdecomposition_gb300 import truss as T
    d = GD.load("fixture")
    p = tmp_path / "g.txt"
    _write_text(p, d["pairs"])
    g, verts = F.read_graph(str(p))
    assert g.columns.is_cuda and g.num_edges == len(d["ref_cols"])
    res = T.truss_decompose(g)
    assert res.kmax == int(d["sg_kmax2"])
    assert res.triangles == int(d["ref_support"].sum()) // 3
