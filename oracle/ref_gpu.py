"""TEST AND BENCH INFRASTRUCTURE ONLY -- the reference's own GPU kernels.

Loads ``oracle/_ref/trusstensor_sm103a.cubin`` (the reference's
``demo_truss/myops/mysrc/hpu_extension/myhpu_extension_kernel.cu``, compiled
unmodified for sm_103a by ``oracle/build.py``) with the CUDA driver API, and
launches its kernels exactly as the reference's launchers do: 512 threads a
block, ceil(rows / 512) blocks, where rows is

* ``segment_add``: output.size(0)                  (kernel.cu:22-26, cpp:8-18);
* ``segment_isin2``: output.size(0)                (kernel.cu:62-79);
* ``segment_isin2tile``: output.size(0) * n_cut    (kernel.cu:117-134);
* ``sub_AllAffectedSupport_not``: e_affect.size(0) (kernel.cu:275-300);
* ``sub_AllAffectedSupport_tilenot``: e_affect.size(0) * n_cut (kernel.cu:548-577).

Those are the operators the reference's ``--cuda`` flow calls
(demo_truss/singlegpu_truss.py:38-64); ``RefKernels`` exposes them under the
``trusstensor`` names so ``tdtdecomposition_gb300.flow`` can run over them
(the reference GPU path on this GPU, timed beside the build's kernels).  The
launches go to torch's current stream (the reference uses the legacy default
stream; with one stream in use the two are equivalent).

In that flow every index the kernels take stays inside its array: the
affected edges never include a peeled edge (a peeled edge's column -1 reads
the mask of vertex V-1, the top-ranked vertex, which has no out-edges and so
is never a peeled edge's tail), and the -1 columns met inside a merge are
compared, never used as an index.

Only bench.py and tests use this module; the product package never does.
"""
import ctypes
import os

from . import build as _build

# entry points of the image (the names ptxas reports for the reference's
# kernels; C++ mangling of their signatures)
_ENTRY = {
    "segment_add": "_Z16segmentAddKernelPKiS0_Pii",
    "segment_isin2": "_Z19checkElementsTwoPtrPKiS0_S0_Pii",
    "segment_isin2tile": "_Z23checkElementsTwoPtrTilePKiS0_S0_iPii",
    "sub_AllAffectedSupport_not": "_Z22AllAffectedSupport_notPKiS0_S0_S0_PKbiPbPii",
    "sub_AllAffectedSupport_tilenot": "_Z26AllAffectedSupport_tilenotPKiS0_S0_S0_iPKbiPbPii",
}
_BLOCK = 512


def image_path():
    return _build.REF_CUBIN


def available():
    return os.path.exists(_build.REF_CUBIN)


class RefKernels:
    """The reference's kernels, launched like its launchers do."""

    def __init__(self, path=None):
        import torch
        path = path or _build.REF_CUBIN
        if not os.path.exists(path):
            raise FileNotFoundError("reference kernel image not built: %s" % path)
        torch.zeros(1, device="cuda")  # the primary context, current on this thread
        cu = ctypes.CDLL("libcuda.so.1")
        cu.cuModuleLoadData.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
        cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [ctypes.c_void_p,
                                                                                 ctypes.POINTER(ctypes.c_void_p),
                                                                                 ctypes.c_void_p]
        self._cu = cu
        with open(path, "rb") as f:
            img = f.read()
        self._img = ctypes.create_string_buffer(img, len(img))
        mod = ctypes.c_void_p()
        self._check(cu.cuModuleLoadData(ctypes.byref(mod), self._img), "cuModuleLoadData")
        self._mod = mod
        self._fn = {}
        for op, name in _ENTRY.items():
            fn = ctypes.c_void_p()
            self._check(cu.cuModuleGetFunction(ctypes.byref(fn), mod, name.encode()), "cuModuleGetFunction " + name)
            self._fn[op] = fn
        self.launches = 0

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError("%s failed: CUresult %d" % (what, rc))

    def _launch(self, op, rows, args):
        import torch
        if rows <= 0:
            return
        vals = []
        for a in args:
            if isinstance(a, torch.Tensor):
                vals.append(ctypes.c_void_p(a.data_ptr()))
            else:
                vals.append(ctypes.c_int(int(a)))
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        stream = torch.cuda.current_stream().cuda_stream
        grid = (rows + _BLOCK - 1) // _BLOCK
        self._check(self._cu.cuLaunchKernel(self._fn[op], grid, 1, 1, _BLOCK, 1, 1, 0, ctypes.c_void_p(stream),
                                            params, None), "cuLaunchKernel " + op)
        self.launches += 1

    # the trusstensor operators (in place, as the reference's)
    def segment_add(self, col_indices, col_ptr, output):
        n = output.shape[0]
        self._launch("segment_add", n, [col_indices, col_ptr, output, n])

    def segment_isin2(self, a_rows, b_col_indices, b_row_ptr, output):
        n = output.shape[0]
        self._launch("segment_isin2", n, [a_rows, b_col_indices, b_row_ptr, output, n])

    def segment_isin2tile(self, a_rows, b_col_indices, b_row_ptr, n_cut, output):
        n = output.shape[0] * int(n_cut)
        self._launch("segment_isin2tile", n, [a_rows, b_col_indices, b_row_ptr, int(n_cut), output, n])

    def sub_AllAffectedSupport_not(self, e_affect, a_rows, b_col_indices, b_row_ptr, mark, l, n_mark, output):
        n = e_affect.shape[0]
        self._launch("sub_AllAffectedSupport_not", n,
                     [e_affect, a_rows, b_col_indices, b_row_ptr, mark, int(l), n_mark, output, n])

    def sub_AllAffectedSupport_tilenot(self, e_affect, a_rows, b_col_indices, b_row_ptr, n_cut, mark, l, n_mark,
                                       output):
        n = e_affect.shape[0] * int(n_cut)
        self._launch("sub_AllAffectedSupport_tilenot", n,
                     [e_affect, a_rows, b_col_indices, b_row_ptr, int(n_cut), mark, int(l), n_mark, output, n])


def k_truss_on_reference_kernels(graph, n_cut, num_v, kernels=None):
    """The `--cuda` flow (tdtdecomposition_gb300.flow.k_truss, the restated
    singlegpu_truss.py:67-158) over the reference's own GPU kernels.  Mutates
    graph like the reference.  Returns (kmax, e_truss, ptr_truss)."""
    from tdtdecomposition_gb300 import flow
    kernels = kernels or RefKernels()
    saved = flow.tt
    flow.tt = kernels
    try:
        return flow.k_truss(graph, n_cut, num_v)
    finally:
        flow.tt = saved
