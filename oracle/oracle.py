"""ctypes wrapper of the C oracle (``oracle/hsolve_oracle.c``).  TEST INFRASTRUCTURE.

The oracle restates the reference HSolve on the CPU.  Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU legs import this module; the
product never does.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libhsolve_oracle.so")
SRC = os.path.join(HERE, "hsolve_oracle.c")

sys.path.insert(0, os.path.join(os.path.dirname(HERE), "moose-core_gb300"))
from moose_gb300.abi import CellModel, HsCellDesc  # noqa: E402


def build(force=False):
    """Compile the oracle with the reference build's FP flags."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "hsolve_oracle.h"))):
        return LIB
    cmd = ["gcc", "-O2", "-std=c99", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB, SRC, "-lm"]
    subprocess.check_call(cmd)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        pd = C.POINTER(C.c_double)
        pu = C.POINTER(C.c_uint32)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.POINTER(HsCellDesc), C.c_uint32, C.c_double, C.c_char_p, C.c_uint32]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_ca_advance.argtypes = [vp, C.c_int]
        L.orc_set_f32_gate_increments.argtypes = [vp, C.c_int]
        L.orc_read_dif.argtypes = [vp, pd]
        L.orc_reinit.argtypes = [vp, C.c_double]
        L.orc_step.argtypes = [vp, C.c_uint32]
        for f in ("orc_n_compt", "orc_n_pool", "orc_n_state"):
            getattr(L, f).restype = C.c_uint32
            getattr(L, f).argtypes = [vp]
        L.orc_hines_index.restype = C.c_uint32
        L.orc_hines_index.argtypes = [vp, C.c_uint32]
        L.orc_model_index.restype = C.c_uint32
        L.orc_model_index.argtypes = [vp, C.c_uint32]
        L.orc_read_vm.argtypes = [vp, pd]
        L.orc_read_ca.argtypes = [vp, pd]
        L.orc_read_state.argtypes = [vp, pd]
        L.orc_read_spikes.restype = C.c_uint32
        L.orc_read_spikes.argtypes = [vp, pu, pd, C.c_uint32]
        L.orc_table_grid.argtypes = [vp, pd]
        L.orc_get_field.restype = C.c_int
        L.orc_get_field.argtypes = [vp, C.c_int, C.c_int, C.c_uint32, pd]
        L.orc_set_field.restype = C.c_int
        L.orc_set_field.argtypes = [vp, C.c_int, C.c_int, C.c_uint32, C.c_double]
        for f in ("orc_add_inject", "orc_add_conc", "orc_add_ica"):
            getattr(L, f).restype = C.c_int
            getattr(L, f).argtypes = [vp, C.c_uint32, C.c_double]
        L.orc_push_event.restype = C.c_int
        L.orc_push_event.argtypes = [vp, C.c_uint32, C.c_double, C.c_double]
        L.orc_add_gkek.restype = C.c_int
        L.orc_add_gkek.argtypes = [vp, C.c_uint32, C.c_double, C.c_double]
        L.orc_passive_create.restype = vp
        L.orc_passive_create.argtypes = [C.c_uint32, pu, pu, pd, pd, pd, pd, pd, C.c_double]
        for f in ("orc_passive_update", "orc_forward", "orc_backward"):
            getattr(L, f).argtypes = [vp]
        L.orc_getA.restype = C.c_double
        L.orc_getA.argtypes = [vp, C.c_uint32, C.c_uint32]
        for f in ("orc_getB", "orc_getVMid", "orc_getV"):
            getattr(L, f).restype = C.c_double
            getattr(L, f).argtypes = [vp, C.c_uint32]
        _lib = L
    return _lib


def _pd(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleCell:
    """One cell stepped by the CPU oracle (HSolve restated)."""

    def __init__(self, model: CellModel, dt, seed=None):
        self.model = model
        self._desc = model.desc()
        err = C.create_string_buffer(256)
        s = model.seed if seed is None else seed
        self.h = lib().orc_create(C.byref(self._desc), s, dt, err, 256)
        if not self.h:
            raise ValueError("oracle setup failed: " + err.value.decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def set_ca_advance(self, v):
        lib().orc_set_ca_advance(self.h, int(v))

    def set_f32_gate_increments(self, on=True):
        """Conditioning probe (not the reference's arithmetic): gate increments
        in FP32, accumulated in FP64, as a mixed-precision solver gates."""
        lib().orc_set_f32_gate_increments(self.h, int(bool(on)))

    def reinit(self, dt):
        lib().orc_reinit(self.h, dt)

    def step(self, n=1):
        lib().orc_step(self.h, int(n))

    def vm(self):
        out = np.empty(self.model.n_compt)
        lib().orc_read_vm(self.h, _pd(out))
        return out

    def ca(self):
        out = np.empty(len(self.model.pool_compt))
        lib().orc_read_ca(self.h, _pd(out))
        return out

    def dif(self):
        """C of each DifShell, bFree of each DifBuffer (0 for an MMPump)."""
        out = np.empty(len(self.model.dif_kind))
        if len(out):
            lib().orc_read_dif(self.h, _pd(out))
        return out

    def state(self):
        out = np.empty(lib().orc_n_state(self.h))
        lib().orc_read_state(self.h, _pd(out))
        return out

    def spikes(self):
        n = lib().orc_read_spikes(self.h, None, None, 0)
        g = np.empty(n, np.uint32)
        t = np.empty(n)
        lib().orc_read_spikes(self.h, g.ctypes.data_as(C.POINTER(C.c_uint32)), _pd(t), n)
        return g, t

    def table_grid(self):
        g = np.empty(6)
        lib().orc_table_grid(self.h, _pd(g))
        return g

    def hines_order(self):
        n = lib().orc_n_compt(self.h)
        return np.array([lib().orc_model_index(self.h, i) for i in range(n)], np.uint32)

    def get(self, kind, field, index):
        out = C.c_double()
        rc = lib().orc_get_field(self.h, kind, field, index, C.byref(out))
        if rc:
            raise IndexError("oracle get_field failed")
        return out.value

    def set(self, kind, field, index, value):
        if lib().orc_set_field(self.h, kind, field, index, float(value)):
            raise IndexError("oracle set_field failed")

    # message destinations (HSolve::addInject, addGkEk, addConc, iCa)
    def add_inject(self, compt, value):
        if lib().orc_add_inject(self.h, int(compt), float(value)):
            raise IndexError("oracle add_inject failed")

    def add_gkek(self, compt, gk, ek):
        if lib().orc_add_gkek(self.h, int(compt), float(gk), float(ek)):
            raise IndexError("oracle add_gkek failed")

    def add_conc(self, chan, conc):
        if lib().orc_add_conc(self.h, int(chan), float(conc)):
            raise IndexError("oracle add_conc failed")

    def add_ica(self, pool, ica):
        if lib().orc_add_ica(self.h, int(pool), float(ica)):
            raise IndexError("oracle add_ica failed")

    def push_events(self, syn, time, weight):
        """SimpleSynHandler::addSpike for each (syn, time, weight), in order."""
        for k, t, w in zip(np.atleast_1d(syn), np.atleast_1d(time), np.atleast_1d(weight)):
            if lib().orc_push_event(self.h, int(k), float(t), float(w)):
                raise IndexError("oracle push_events failed")


class OraclePassive:
    """HinesMatrix/HSolvePassive on a tree given in Hines order (unit tests)."""

    def __init__(self, children, Ra, Rm, Cm, Em, V, dt):
        n = len(children)
        off = np.zeros(n + 1, np.uint32)
        for i, c in enumerate(children):
            off[i + 1] = off[i] + len(c)
        idx = np.array([x for c in children for x in c] or [0], np.uint32)
        self._keep = [np.ascontiguousarray(a, np.float64) for a in (Ra, Rm, Cm, Em, V)]
        pu = C.POINTER(C.c_uint32)
        self.n = n
        self.h = lib().orc_passive_create(n, off.ctypes.data_as(pu), idx.ctypes.data_as(pu),
                                          *[_pd(a) for a in self._keep], dt)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def update(self):
        lib().orc_passive_update(self.h)

    def forward(self):
        lib().orc_forward(self.h)

    def backward(self):
        lib().orc_backward(self.h)

    def A(self):
        n = self.n
        return np.array([[lib().orc_getA(self.h, i, j) for j in range(n)] for i in range(n)])

    def B(self):
        return np.array([lib().orc_getB(self.h, i) for i in range(self.n)])

    def VMid(self):
        return np.array([lib().orc_getVMid(self.h, i) for i in range(self.n)])

    def V(self):
        return np.array([lib().orc_getV(self.h, i) for i in range(self.n)])
