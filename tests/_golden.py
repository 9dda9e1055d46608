"""Loading of the golden fixtures (tests/golden/*.npz) shared by the tests."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    if "pairs" not in d:
        from tdtdecomposition_gb300 import generators as G
        if name == "er_4096_65536":
            s, t = G.er_edges(4096, 65536, seed=0)
            d["pairs"] = np.stack([s, t], 1).astype(np.int32)
    return d


def truss_from_levels(e_truss, ptr_truss, E):
    t = np.full(E, 2, np.int32)
    for lv in range(len(ptr_truss) - 1):
        t[e_truss[ptr_truss[lv]:ptr_truss[lv + 1]]] = lv + 3
    return t


def edge_set(rows, cols):
    return set(zip(np.asarray(rows).tolist(), np.asarray(cols).tolist()))
