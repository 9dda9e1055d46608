"""The C-ABI library loads and exports every entry point include/*.h
declares (no compute call: this runs without a GPU)."""
import glob
import os
import re
import subprocess

import pytest

from tdtdecomposition_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"\b(tdt_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = _declared()
    assert "tdt_truss_decompose" in names and "tdt_segment_isin2tile" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.lib_path()], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\sT\s(tdt_\w+)", out))
    missing = [n for n in _declared() if n not in exported]
    assert not missing, missing
    for n in _declared():
        assert hasattr(lib, n)


def test_python_binding_covers_header():
    assert set(_declared()) <= set(_lib.exported_names()) | {"tdt_gen_rmat", "tdt_gen_ba", "tdt_splitmix64"}


def test_status_strings(lib):
    assert lib.tdt_status_string(0) == b"ok"
    assert b"timed out" in lib.tdt_status_string(4)
    assert lib.tdt_version() >= 100


def test_workspace_query_is_pure_host(lib):
    a = lib.tdt_decompose_workspace_bytes(1000, 10000)
    b = lib.tdt_decompose_workspace_bytes(1000, 20000)
    assert 0 < a < b
    assert lib.tdt_decompose_workspace_bytes(0, 0) > 0


def test_built_for_sm103a_only():
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_noalloc_scratch_holds_its_size_limit(lib):
    """tdt_triangle_count_noalloc accepts graphs up to 2^18 vertices and 2^18
    edges; the workspace of that corner must fit its fixed 40 MiB scratch."""
    assert lib.tdt_decompose_workspace_bytes(1 << 18, 1 << 18) <= 40 << 20
