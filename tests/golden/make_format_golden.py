"""Golden files for the on-disk formats, made by the reference's own code (run
where the reference tree exists; the outputs are committed and the tests never
read the reference tree):

* fmt_csr_pairs.npy and fmt_csr_ref/{csr_vlist.bin, csr_elist.bin}: the
  reference's converter demo_truss/test/txt_to_csrcoo.cpp (compiled here with
  g++) run on a seeded edge list (tab-separated text, no header);
* fmt_ref_csrcoo.pth: the README fixture graph (tests/golden/fixture.npz)
  saved by torch.save as an instance of the reference's own class
  src/type/CSRCOO.py:CSRCOO (int32 row_ptr, as read_prepro_save writes it).

Usage: python tests/golden/make_format_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("TDT_REFERENCE_ROOT", "/root/reference")


def csr_tool():
    rng = np.random.default_rng(5)
    pairs = (rng.integers(0, 300, size=(2000, 2)) * 3 + 1).astype(np.int64)
    np.save(os.path.join(HERE, "fmt_csr_pairs.npy"), pairs)
    out = os.path.join(HERE, "fmt_csr_ref")
    os.makedirs(out, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        txt = os.path.join(tmp, "g.txt")
        with open(txt, "w") as f:
            for a, b in pairs:
                f.write("%d\t%d\n" % (a, b))
        exe = os.path.join(tmp, "txt_to_csrcoo")
        subprocess.run(["g++", "-O2", "-o", exe, os.path.join(REF, "demo_truss/test/txt_to_csrcoo.cpp")],
                       check=True)
        subprocess.run([exe, txt, out], check=True, capture_output=True)


def ref_pth():
    d = np.load(os.path.join(HERE, "fixture.npz"))
    code = r"""
import sys, numpy as np, torch
sys.path.insert(0, %r)
from src.type.CSRCOO import CSRCOO
d = np.load(%r)
g = CSRCOO(columns=torch.as_tensor(d["ref_cols"], dtype=torch.int32),
           row_ptr=torch.as_tensor(d["ref_rp"], dtype=torch.int32),
           rows=torch.as_tensor(d["ref_rows"], dtype=torch.int32))
torch.save(g, %r)
""" % (REF, os.path.join(HERE, "fixture.npz"), os.path.join(HERE, "fmt_ref_csrcoo.pth"))
    subprocess.run([sys.executable, "-c", code], check=True)
    return d


if __name__ == "__main__":
    csr_tool()
    ref_pth()
    print("written under", HERE)
