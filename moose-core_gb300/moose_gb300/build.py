"""Build of the native library ``libmoose_gb300.so`` (CUDA for sm_103a + C++).

Translation units:
  * ``hs_fp64.cu``  -- FP64 kernels, ``--fmad=false`` so every a*b+c stays two
    IEEE roundings, exactly as the reference CPU code computes it;
  * ``hs_mixed.cu`` -- the mixed-precision batched kernel (FMA contraction on);
  * ``hs_cell.cu``  -- device-arena upload;
  * ``hs_noalloc.cu`` -- inject writes from fixed storage (no allocation);
  * ``hs_plan.cpp``, ``hs_api.cpp``, ``hs_batch_api.cpp`` -- host setup and
    the C ABI, ``-ffp-contract=off`` for the same reason.
The library is built in-tree under ``moose_gb300/_lib`` (git-ignored).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(PKG), "csrc")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libmoose_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _cuda_include():
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(_nvcc()))), "include")


UNITS = {
    "hs_fp64.cu": ["--fmad=false"],
    "hs_mixed.cu": [],
    "hs_cell.cu": ["--fmad=false"],
    "hs_noalloc.cu": [],
    "hs_plan.cpp": None,
    "hs_api.cpp": None,
    "hs_batch_api.cpp": None,
}


def _sources():
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(os.path.dirname(PKG)), "include", "moose_gb300.h"))
    return deps


def _compile(unit, extra):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT, unit + ".o")
    if extra is None:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
               "-Wno-unused-function", "-I" + _cuda_include(), "-c", src, "-o", obj]
    else:
        cmd = [_nvcc()] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                                  "-Xcompiler", "-ffp-contract=off"] + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(force=False, verbose=False):
    """Compile every unit for sm_103a and link the shared library."""
    os.makedirs(OUT, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in _sources())
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    units = {u: e for u, e in UNITS.items() if os.path.exists(os.path.join(CSRC, u))}
    with cf.ThreadPoolExecutor(len(units)) as ex:
        objs = list(ex.map(lambda kv: _compile(*kv), units.items()))
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
