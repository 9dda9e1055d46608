"""Digests of the oracle's decomposition of the large benchmark graphs.

The oracle (oracle/tdt_oracle.c: the `--cuda` flow of
demo_truss/singlegpu_truss.py:67-158 over the restated operators, OpenMP)
needs minutes on these graphs, so it runs here once and its outputs are
committed as SHA-256 digests of their little-endian bytes
(tests/golden/fullsize_digests.json):

* rmat_s22: R-MAT scale 22, edge factor 16, (a,b,c,d) = (.57,.19,.19,.05),
  seed 1 -- the graph the benchmark times;
* chung_lu_18, chung_lu_20: Chung-Lu n = 2^18 and 2^20, exponent 2.1, mean
  degree 40, degree cap 2^20, seed 2 -- the skewed family at sizes the
  oracle finishes in minutes.

Each case records the CSR it was run on (digests of columns and int64
row_ptr, so the GPU test can show it preprocessed the same graph), V, E, the
triangle count, kmax, and the digests of per-edge support, truss numbers,
e_truss and ptr_truss.  The graphs come from the host generators
(tdtdecomposition_gb300/generators.py, the same draw stream as the device
generators) and the oracle's preprocessing (stable (degree, id) rank).

Usage: python tests/golden/make_fullsize_digests.py [case ...]
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import oracle as O  # noqa: E402
from tdtdecomposition_gb300 import generators as G  # noqa: E402

OUT = os.path.join(HERE, "fullsize_digests.json")
N_CUT = 2

CASES = {
    "rmat_s22": dict(kind="rmat", scale=22, edge_factor=16, seed=1),
    "chung_lu_18": dict(kind="chung_lu", log2n=18, gamma=2.1, mean_degree=40.0, max_degree=1 << 20, seed=2),
    "chung_lu_20": dict(kind="chung_lu", log2n=20, gamma=2.1, mean_degree=40.0, max_degree=1 << 20, seed=2),
}


def sha(a, dtype):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.dtype(dtype).newbyteorder("<")).tobytes()).hexdigest()


def edges(p):
    if p["kind"] == "rmat":
        return G.rmat_edges(p["scale"], p["edge_factor"] << p["scale"], seed=p["seed"])
    return G.chung_lu_edges(1 << p["log2n"], p["gamma"], p["mean_degree"], p["max_degree"], seed=p["seed"])


def run(name):
    p = CASES[name]
    t0 = time.time()
    s, d = edges(p)
    rows, cols, rp, verts = O.preprocess(np.stack([s, d], 1))
    del s, d
    V, E = len(verts), len(cols)
    t1 = time.time()
    sup = O.support(rows, cols, rp.astype(np.int32), 1)
    tri = int(sup.sum(dtype=np.int64)) // 3
    kmax, et, pt, truss = O.k_truss(rows, cols, O.tiling_row_ptr(rows, cols, V, N_CUT), V, N_CUT)
    t2 = time.time()
    rec = dict(params=p, n_cut=N_CUT, V=V, E=E, triangles=tri, kmax=kmax, n_etruss=int(len(et)),
               n_ptr=int(len(pt)),
               sha256=dict(columns=sha(cols, np.int32), row_ptr=sha(rp, np.int64), support=sha(sup, np.int32),
                           truss=sha(truss, np.int32), e_truss=sha(et, np.int32), ptr_truss=sha(pt, np.int32)),
               oracle_seconds=dict(preprocess=round(t1 - t0, 1), decompose=round(t2 - t1, 1),
                                   threads=O.num_threads()))
    print(name, json.dumps(rec), flush=True)
    return rec


def main(names):
    have = json.load(open(OUT)) if os.path.exists(OUT) else {}
    for n in names:
        have[n] = run(n)
        with open(OUT, "w") as f:
            json.dump(have, f, indent=1, sort_keys=True)
            f.write("\n")


if __name__ == "__main__":
    main(sys.argv[1:] or list(CASES))
