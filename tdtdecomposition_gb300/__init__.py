"""GB300-native (sm_103a) truss decomposition: the TDT hot path
(support / triangle counting, level-synchronous peeling, k-truss search)
behind the reference's ``trusstensor`` operator surface.

* :mod:`.trusstensor` - drop-in operators (same names and semantics);
* :mod:`.truss`       - device-resident whole-path API;
* :mod:`.flow`        - the reference's host-driven flow over the drop-in ops;
* :mod:`.graph`       - the CSRCOO container;
* :mod:`.generators`  - seeded synthetic workloads.

The native library is built in-tree (``python -m tdtdecomposition_gb300.build``);
there is no CPU fallback.
"""
from .graph import CSRCOO, tiling_row_ptr  # noqa: F401

__version__ = "0.1.0"


def __getattr__(name):
    if name in ("truss_decompose", "ktruss_search", "triangle_count", "TrussResult", "Workspace"):
        from . import truss
        return getattr(truss, name)
    raise AttributeError(name)
