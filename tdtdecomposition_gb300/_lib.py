"""ctypes binding of libtdt_gb300.so (the C ABI in include/tdt_gb300.h).

The library is built in-tree by ``tdtdecomposition_gb300.build``.  There is no
CPU fallback: when the library is missing or cannot be loaded, every
operation raises.
"""
import ctypes
import os
import threading

from . import build as _build

_I32P = ctypes.c_void_p
_lock = threading.Lock()
_lib = None

c_i64 = ctypes.c_int64
c_i32 = ctypes.c_int32
c_ptr = ctypes.c_void_p
c_size = ctypes.c_size_t

# (name, restype, argtypes)
_SIGS = [
    ("tdt_status_string", ctypes.c_char_p, [ctypes.c_int]),
    ("tdt_last_error", ctypes.c_char_p, []),
    ("tdt_version", ctypes.c_int, []),
    ("tdt_launch_count", ctypes.c_ulonglong, []),
    ("tdt_profile_start", ctypes.c_int, [ctypes.c_int]),
    ("tdt_profile_stop", ctypes.c_int, [c_ptr, c_ptr]),
    ("tdt_peel_clock", ctypes.c_int, [c_ptr, c_ptr, c_ptr]),
    ("tdt_set_support_caps", None, [ctypes.c_int, ctypes.c_int]),
    ("tdt_set_vector_walk", None, [ctypes.c_int]),
    ("tdt_set_bulk_staging", None, [ctypes.c_int]),
    ("tdt_set_peel_grid", None, [ctypes.c_int]),
    ("tdt_set_peel_deadline_ns", None, [ctypes.c_longlong]),
    ("tdt_set_ktruss_batch_caps", None, [ctypes.c_longlong, ctypes.c_longlong]),
    ("tdt_set_peel_dynamic_min", None, [ctypes.c_longlong]),
    ("tdt_test_barrier_timeout", ctypes.c_int, [c_ptr, ctypes.c_longlong, c_ptr]),
    ("tdt_segment_add", ctypes.c_int, [c_ptr, c_i64, c_ptr, c_ptr, c_i64, c_ptr]),
    ("tdt_segment_isin2", ctypes.c_int, [c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_i64, c_ptr]),
    ("tdt_segment_isin2tile", ctypes.c_int, [c_ptr, c_ptr, c_ptr, c_i64, c_i32, c_ptr, c_i64, c_ptr]),
    ("tdt_sub_all_affected_support", ctypes.c_int,
     [c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_i32, c_ptr, c_ptr, c_i64, c_ptr]),
    ("tdt_sub_all_affected_support_tile", ctypes.c_int,
     [c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_i64, c_i32, c_ptr, c_i32, c_ptr, c_ptr, c_i64, c_ptr]),
    ("tdt_sub_all_affected_support_not", ctypes.c_int,
     [c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_i32, c_ptr, c_ptr, c_i64, c_ptr]),
    ("tdt_sub_all_affected_support_tilenot", ctypes.c_int,
     [c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_i64, c_i32, c_ptr, c_i32, c_ptr, c_ptr, c_i64, c_ptr]),
    ("tdt_sub_all_affected_support_notwin", ctypes.c_int,
     [c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_i32, c_ptr, c_ptr, c_i32, c_ptr, c_ptr, c_ptr,
      c_i64, c_ptr]),
    ("tdt_sub_all_affected_support_tilenotwin", ctypes.c_int,
     [c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_i64, c_i32, c_ptr, c_i32, c_ptr, c_ptr, c_i32, c_ptr, c_ptr,
      c_ptr, c_i64, c_ptr]),
    ("tdt_segment_isin2_k", ctypes.c_int, [c_ptr, c_ptr, c_ptr, c_i64, c_i32, c_ptr, c_i64, c_ptr]),
    ("tdt_segment_isin2tile_k", ctypes.c_int, [c_ptr, c_ptr, c_ptr, c_i64, c_i32, c_i32, c_ptr, c_i64, c_ptr]),
    ("tdt_sub_affected_support", ctypes.c_int, [c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_i64, c_ptr]),
    ("tdt_sub_affected_support_tile", ctypes.c_int,
     [c_ptr, c_ptr, c_ptr, c_i64, c_i32, c_ptr, c_ptr, c_i64, c_ptr]),
    ("tdt_segment_isinis_m", ctypes.c_int, [c_ptr, c_i64, c_ptr, c_ptr, c_i64, c_ptr, c_i64, c_ptr, c_ptr, c_ptr]),
    ("tdt_segment_isinmm", ctypes.c_int, [c_ptr, c_i64, c_ptr, c_i64, c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_ptr]),
    ("tdt_sub_suppport_affect", ctypes.c_int,
     [c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_i32, c_ptr]),
    ("tdt_peeling_undirect", ctypes.c_int,
     [c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_ptr, c_i32, c_i64,
      c_ptr]),
    ("tdt_peeling_undirect_tile", ctypes.c_int,
     [c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_ptr, c_i32, c_i32,
      c_i64, c_ptr]),
    ("tdt_peeling_direct_oo", ctypes.c_int,
     [c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_ptr, c_i32, c_i64, c_ptr]),
    ("tdt_peeling_direct_tile_oo", ctypes.c_int,
     [c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_ptr, c_i32, c_i32, c_i64, c_ptr]),
    ("tdt_peeling_direct_ii", ctypes.c_int,
     [c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_ptr, c_i32, c_i64, c_ptr]),
    ("tdt_peeling_direct_tile_ii", ctypes.c_int,
     [c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_ptr, c_i32, c_i32, c_i64, c_ptr]),
    ("tdt_peeling_direct_oi", ctypes.c_int,
     [c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_ptr, c_i32, c_i64,
      c_ptr]),
    ("tdt_peeling_direct_tile_oi", ctypes.c_int,
     [c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_ptr, c_i32, c_i32,
      c_i64, c_ptr]),
    ("tdt_preprocess_workspace_bytes", c_size, [c_i64, c_i64]),
    ("tdt_preprocess", ctypes.c_int,
     [c_ptr, c_ptr, c_i64, c_i64, c_ptr, c_i32, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_size, c_ptr]),
    ("tdt_decompose_workspace_bytes", c_size, [c_i64, c_i64]),
    ("tdt_truss_decompose", ctypes.c_int,
     [c_ptr, c_ptr, c_ptr, c_i64, c_i64, c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_size, c_ptr]),
    ("tdt_triangle_count", ctypes.c_int, [c_ptr, c_ptr, c_i64, c_i64, c_ptr, c_ptr, c_ptr, c_size, c_ptr]),
    ("tdt_triangle_count_noalloc", ctypes.c_int, [c_ptr, c_ptr, c_i64, c_i64, c_ptr, c_ptr, c_ptr]),
    ("tdt_ktruss_search", ctypes.c_int,
     [c_ptr, c_ptr, c_ptr, c_i64, c_i64, c_i32, c_ptr, c_ptr, c_ptr, c_size, c_ptr]),
]


class TdtError(RuntimeError):
    """A libtdt_gb300 call returned a non-zero status."""

    def __init__(self, status, where, detail=""):
        self.status = status
        super().__init__("%s failed: %s%s" % (where, status_string(status), (" (%s)" % detail) if detail else ""))


def lib_path():
    return _build.LIB


def load(build_if_missing=False):
    """Load (and with build_if_missing, first build) libtdt_gb300.so."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise ImportError("libtdt_gb300.so is not built (expected at %s); run "
                                  "`python -m tdtdecomposition_gb300.build` or __graft_entry__.build()" % path)
            _build.build()
        L = ctypes.CDLL(path)
        for name, res, args in _SIGS:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_names():
    return [n for n, _, _ in _SIGS]


def status_string(status):
    try:
        return load().tdt_status_string(int(status)).decode()
    except Exception:  # library not loadable: still give a message
        return "status %d" % int(status)


def check(status, where):
    if status != 0:
        detail = load().tdt_last_error().decode(errors="replace")
        raise TdtError(status, where, detail)
