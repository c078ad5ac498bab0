"""The C++ HSolve mirror (moose-core_gb300/cpp/hsolve_gpu.hpp) over the C ABI.

tests/cpp/hsolve_cpp_shim.cpp is compiled here with g++ against the header
and libmoose_gb300.so.  Without a GPU: the header compiles and links, and
the class keeps the reference's field rules (dt >= 0, caAdvance 0 or 1,
"Must set 'dt' first", an error for any field access without a solver).
On the GPU: a run driven through the class -- field writes, message
destinations, process -- gives Vm and Ca bit-identical to the same calls
made through the Python mirror and to the oracle.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from moose_gb300 import _native, models
from moose_gb300.abi import FIELDS, HS_KIND_CHAN, HS_KIND_COMPT, HsCellDesc
from moose_gb300.hsolve import HSolve
from oracle import OracleCell

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT = os.path.join(HERE, "cpp", "_build")


def shim():
    _native.load()
    libdir = os.path.dirname(_native.lib_path())
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "libhsolve_cpp_shim.so")
    src = os.path.join(HERE, "cpp", "hsolve_cpp_shim.cpp")
    hdr = os.path.join(REPO, "moose-core_gb300", "cpp", "hsolve_gpu.hpp")
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(src), os.path.getmtime(hdr),
                                                            os.path.getmtime(_native.lib_path())):
        cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-fPIC", "-shared", "-o", so, src,
               "-I", os.path.join(REPO, "include"), "-I", os.path.join(REPO, "moose-core_gb300", "cpp"),
               "-L", libdir, "-lmoose_gb300", "-Wl,-rpath," + libdir]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
    L = C.CDLL(so)
    pd = C.POINTER(C.c_double)
    L.hsolve_cpp_run.argtypes = [C.POINTER(HsCellDesc), C.c_uint32, C.c_double, C.c_uint32, C.c_uint32,
                                 C.c_uint32, pd, pd, C.c_char_p, C.c_uint32]
    L.hsolve_cpp_errors.argtypes = [C.POINTER(HsCellDesc)]
    return L


def test_header_compiles_and_keeps_the_field_rules():
    L = shim()
    m = models.config1_cell(n_cable=5)
    d = m.desc()
    assert L.hsolve_cpp_errors(C.byref(d)) == 0


def _libm_free_cells():
    rng = np.random.default_rng(11)
    parent, d, L = models.branched_morphology(rng, 80, 0.6, 4)
    m = models.active_cell(parent, d, L, inject=0.5e-9, gca=10.0, gkca=0.0)
    for k in list(vars(m)):
        if k.startswith("c2d_"):
            setattr(m, k, getattr(m, k)[:0])
    m.gates2d = []
    return [models.config1_cell(n_cable=60, inject=0.4e-9), m]


@pytest.mark.gpu
@pytest.mark.parametrize("which", [0, 1])
def test_cpp_run_matches_python_mirror_and_oracle(which):
    L = shim()
    m = _libm_free_cells()[which]
    dt, n = 25e-6, 1200
    n_c, n_p = m.n_compt, len(m.pool_compt)
    d = m.desc()
    vm = np.empty(n_c)
    ca = np.empty(max(n_p, 1))
    err = C.create_string_buffer(256)
    pd = C.POINTER(C.c_double)
    rc = L.hsolve_cpp_run(C.byref(d), m.seed, dt, n_c, n_p, n, vm.ctypes.data_as(pd), ca.ctypes.data_as(pd),
                          err, 256)
    assert rc == 0, err.value
    # the same calls through the Python mirror and the oracle
    h = HSolve(m, dt=dt)
    h.target = m.seed
    h.reinit(dt)
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    h.process(n // 2)
    oc.step(n // 2)
    em_c = 1 if n_c > 1 else 0
    for s in (h, oc):
        setf = s._set if s is h else s.set
        setf(HS_KIND_COMPT, FIELDS["inject"], 0, 0.3e-9)
        s.add_inject(n_c - 1, 0.1e-9)
        setf(HS_KIND_CHAN, FIELDS["modulation"], 0, 1.2)
        setf(HS_KIND_CHAN, FIELDS["modulation"], 1, 0.0)
        setf(HS_KIND_COMPT, FIELDS["Em"], em_c, -0.07)
        if n_p:
            s.add_ica(0, 1e-12)
    h.process(n - n // 2)
    oc.step(n - n // 2)
    assert np.array_equal(vm, h.vm())
    assert np.array_equal(vm, oc.vm())
    if n_p:
        assert np.array_equal(ca[:n_p], h.ca())
        assert np.array_equal(ca[:n_p], oc.ca())
