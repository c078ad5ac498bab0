#!/usr/bin/env python3
"""Build recipe for the unmodified reference MOOSE (pymoose) from its own sources.

Test infrastructure only.  This script compiles the reference C++ sources where
they lie (``$MOOSE_REF_SRC``, default ``/root/reference``) with plain ``g++``
and links them into a Python extension under ``oracle/_ref/moose/``.  It does
not run the reference's own build system (meson): the per-directory source
lists are read out of each ``<dir>/meson.build`` file and compiled directly.

Differences from the reference's meson recipe, and why:
  * no ``-DUSE_GSL`` / ``-DUSE_HDF5``: GSL and HDF5 are absent here.  Every
    GSL use is ``#ifdef USE_GSL``-guarded, except ``ksolve/SteadyStateGsl.cpp``
    which is left out (chemical steady-state solver, not on the HSolve path).
  * ``-ffp-contract=off``: keep ``a*b+c`` as two rounded operations, so the
    reference's FP64 arithmetic is the plain IEEE sequence the oracle and the
    GPU drop-in restate.
  * the MOOSE-side binding of the GPU solver
    (``moose-core_gb300/cpp/moose_hsolve_bridge.cpp``: an HSolve's setup
    vectors -> ``HsCellDesc``) is compiled against these sources and linked
    into the extension, as a maintainer adding the drop-in to MOOSE would;
    it only adds exported functions (``hsb_*``) and changes no behaviour,
    and the tests call it on HSolves built by the reference's own pymoose.
  * unit tests: a second object set compiled with ``-DDO_UNIT_TESTS`` is not
    needed; the passive-solver known-answer harness (``ref_passive_harness.cpp``)
    links the reference's own HinesMatrix/HSolvePassive objects directly.

Outputs (git-ignored): ``oracle/_ref/obj/**.o``, ``oracle/_ref/libmooseref.a``,
``oracle/_ref/moose/_moose*.so`` plus a copy of the reference's pure-Python
``moose`` package next to it, and ``oracle/_ref/ref_passive_harness``.

Usage:  python oracle/build_ref.py [-j N]
"""
import argparse
import concurrent.futures as cf
import os
import re
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REPO = os.path.dirname(HERE)
BRIDGE = os.path.join(REPO, "moose-core_gb300", "cpp", "moose_hsolve_bridge.cpp")
# The one place that names where the reference sources lie: MOOSE_REF_SRC,
# else the checkout this recipe was written against.  Every other script
# that reads reference files takes the path from here (source_dir()).
SRC = os.environ.get("MOOSE_REF_SRC", "/root/reference")


def source_dir(required=True):
    """The reference source tree, or None (required=False) / SystemExit
    with a message (required=True) when it is not there."""
    if os.path.isdir(SRC):
        return SRC
    if required:
        raise SystemExit("reference sources not found at %s (set MOOSE_REF_SRC)" % SRC)
    return None

# Sub-libraries linked whole into _moose (reference meson.build, `sublibs`).
SUBDIRS = [
    "external/libsoda", "external/fmt", "basecode", "biophysics", "builtins",
    "device", "diffusion", "examples", "hsolve", "intfire", "kinetics",
    "ksolve", "mesh", "mpi", "msg", "pybind11", "randnum", "scheduling",
    "shell", "signeur", "synapse", "utility",
]
EXCLUDE = {
    "ksolve/SteadyStateGsl.cpp",      # GSL-only translation unit
}

CXXFLAGS = [
    "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-fvisibility=hidden",
    "-w", '-DMOOSE_VERSION="4.1.0"', '-DCOMPILER_STRING="gcc"',
]


def sources():
    out = []
    seen = set()
    for d in SUBDIRS:
        mb = os.path.join(SRC, d, "meson.build")
        # drop meson comments: commented-out entries are not part of the build
        text = "\n".join(l.split("#", 1)[0] for l in open(mb).read().splitlines())
        for name in re.findall(r"'([^']+\.(?:cpp|cc))'", text):
            rel = os.path.normpath(os.path.join(d, name))
            if rel in EXCLUDE or rel in seen:
                continue
            seen.add(rel)
            out.append(rel)
    return out


def includes():
    import pybind11
    return [
        "-I" + os.path.join(SRC, "external/fmt/include"),
        "-I" + os.path.join(SRC, "external/libsoda"),
        "-I" + os.path.join(SRC, "external/exprtk"),
        "-I" + os.path.join(SRC),
        "-I" + pybind11.get_include(),
        "-I" + sysconfig.get_paths()["include"],
    ]


def compile_one(rel, inc):
    src = os.path.join(SRC, rel)
    obj = os.path.join(OUT, "obj", rel + ".o")
    os.makedirs(os.path.dirname(obj), exist_ok=True)
    if os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src):
        return obj, None
    cmd = ["g++"] + CXXFLAGS + inc + ["-I" + os.path.dirname(src), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, r.stderr[-4000:]
    return obj, None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("-j", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--keep-objects", action="store_true")
    args = ap.parse_args()
    if not os.path.isdir(SRC):
        print("reference sources not found at", SRC, file=sys.stderr)
        return 2
    os.makedirs(OUT, exist_ok=True)
    inc = includes()
    srcs = sources()
    objs, errors = [], []
    with cf.ThreadPoolExecutor(args.j) as ex:
        for obj, err in ex.map(lambda s: compile_one(s, inc), srcs):
            objs.append(obj)
            if err:
                errors.append((obj, err))
    pym_obj, err = compile_one("pybind11/pymoose.cpp", inc)
    if err:
        errors.append((pym_obj, err))
    bridge_obj = os.path.join(OUT, "obj", "moose_hsolve_bridge.o")
    r = subprocess.run(["g++"] + CXXFLAGS + inc + ["-I" + os.path.join(REPO, "include"), "-c", BRIDGE,
                        "-o", bridge_obj], capture_output=True, text=True)
    if r.returncode != 0:
        errors.append((bridge_obj, r.stderr[-4000:]))
    if errors:
        for obj, err in errors:
            print("FAILED", obj, "\n", err, file=sys.stderr)
        return 1
    lib = os.path.join(OUT, "libmooseref.a")
    if os.path.exists(lib):
        os.remove(lib)
    subprocess.check_call(["ar", "rcs", lib] + objs)
    pkg = os.path.join(OUT, "moose")
    if os.path.isdir(pkg):
        shutil.rmtree(pkg)
    shutil.copytree(os.path.join(SRC, "python", "moose"), pkg)
    ext = os.path.join(pkg, "_moose" + sysconfig.get_config_var("EXT_SUFFIX"))
    subprocess.check_call(
        ["g++", "-shared", "-o", ext, pym_obj, bridge_obj, "-Wl,--whole-archive", lib,
         "-Wl,--no-whole-archive", "-lpthread"])
    rd = os.path.join(OUT, "rdesigneur")
    if os.path.isdir(rd):
        shutil.rmtree(rd)
    shutil.copytree(os.path.join(SRC, "python", "rdesigneur"), rd)
    harness = os.path.join(HERE, "ref_passive_harness.cpp")
    if os.path.exists(harness):
        subprocess.check_call(
            ["g++"] + CXXFLAGS[:3] + ["-fPIC", "-w"] + inc +
            ["-I" + os.path.join(SRC, "hsolve"), harness, "-o",
             os.path.join(OUT, "ref_passive_harness"), lib, "-lpthread"])
    if not args.keep_objects:
        # objects and the archive are only needed to relink; the extension and
        # the harness are what the tests use
        shutil.rmtree(os.path.join(OUT, "obj"), ignore_errors=True)
        os.remove(lib)
    print("built", ext)
    return 0


if __name__ == "__main__":
    sys.exit(main())
