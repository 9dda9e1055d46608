"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles ``tdt_oracle.c`` (the C/OpenMP restatement of the
  reference algorithm) into ``oracle/_build/libtdt_oracle.so``.
* ``build_ref()`` compiles the reference's own OpenMP operator file
  (``demo_truss/myops/mysrc/hpu_extension/myhpu_extension_opmp.cpp``) where it
  lies in the mounted reference tree, together with ``ref_shim.cpp`` (C entry
  points over its C++ functions), into ``oracle/_ref/libtdt_ref.so``.  It runs
  only where the reference tree exists; nothing else reads that tree.

* ``build_ref_cubin()`` compiles the reference's own CUDA kernel file
  (``demo_truss/myops/mysrc/hpu_extension/myhpu_extension_kernel.cu``),
  unmodified, for sm_103a into a device-only image
  ``oracle/_ref/trusstensor_sm103a.cubin``; ``oracle/ref_gpu.py`` loads it
  with the CUDA driver API and launches its kernels the way the reference's
  launchers do (the reference GPU path, timed by bench.py beside the build's
  own kernels).  Like ``build_ref()`` it runs only where the reference tree
  exists.

None of these is part of the product; the package never imports them.
"""
import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libtdt_oracle.so")
REF_SO = os.path.join(REF_DIR, "libtdt_ref.so")
REFERENCE_ROOT = os.environ.get("TDT_REFERENCE_ROOT", "/root/reference")
REF_OPMP = os.path.join(REFERENCE_ROOT, "demo_truss/myops/mysrc/hpu_extension/myhpu_extension_opmp.cpp")
REF_KERNELS = os.path.join(REFERENCE_ROOT, "demo_truss/myops/mysrc/hpu_extension/myhpu_extension_kernel.cu")
REF_CUBIN = os.path.join(REF_DIR, "trusstensor_sm103a.cubin")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    src = os.path.join(HERE, "tdt_oracle.c")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or _stale(ORACLE_SO, [src]):
        tmp = ORACLE_SO + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11",
                               "-o", tmp, src])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(force=False):
    """Compile the reference's OpenMP operators; returns the .so path or None
    when the reference tree is not present."""
    if not os.path.exists(REF_OPMP):
        return REF_SO if os.path.exists(REF_SO) else None
    shim = os.path.join(HERE, "ref_shim.cpp")
    os.makedirs(REF_DIR, exist_ok=True)
    if not (force or _stale(REF_SO, [shim, REF_OPMP])):
        return REF_SO
    from torch.utils.cpp_extension import include_paths
    incs = []
    for p in include_paths() + [sysconfig.get_paths()["include"]]:
        incs += ["-I", p]
    tmp = REF_SO + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c++17",
                           "-w"] + incs + ["-o", tmp, REF_OPMP, shim])
    os.replace(tmp, REF_SO)
    return REF_SO


def build_ref_cubin(force=False):
    """Compile the reference's CUDA kernels for sm_103a into a device-only
    image; returns its path, or None when neither the reference tree nor an
    earlier image is present."""
    if not os.path.exists(REF_KERNELS):
        return REF_CUBIN if os.path.exists(REF_CUBIN) else None
    os.makedirs(REF_DIR, exist_ok=True)
    if not (force or _stale(REF_CUBIN, [REF_KERNELS])):
        return REF_CUBIN
    from torch.utils.cpp_extension import include_paths
    incs = []
    for p in include_paths() + [sysconfig.get_paths()["include"]]:
        incs += ["-I", p]
    nvcc = os.environ.get("NVCC") or "nvcc"
    tmp = REF_CUBIN + ".tmp%d" % os.getpid()
    subprocess.check_call([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-w"]
                          + incs + ["-o", tmp, REF_KERNELS])
    os.replace(tmp, REF_CUBIN)
    return REF_CUBIN


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
    print(build_ref_cubin(force="--force" in sys.argv))
