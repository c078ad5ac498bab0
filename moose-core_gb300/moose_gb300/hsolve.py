"""Host-side mirror of MOOSE's ``HSolve`` class for one cell (the drop-in).

Field names and meanings follow ``hsolve/HSolve.cpp:37-193``: ``dt`` (default
50e-6 s, used for the matrix at setup), ``target`` (setting it runs setup from
the seed compartment, as ``HSolve::setPath``), ``caAdvance``, and the table
grid ``vMin/vMax/vDiv/caMin/caMax/caDiv`` (recomputed from the gates at setup;
user values only read back).  ``reinit(dt)`` and ``process(n)`` are the
clock's tick-6 calls.  Zombie field access goes through ``compartment(i)``,
``channel(i)``, ``pool(i)``, ``chan2d(i)`` and ``synchan(i)`` with MOOSE's
field names (Vm, Cm, Em, Rm, Ra, initVm, Im, inject; Gbar, Ek, Gk, Ik, X, Y,
Z, instant, modulation; Ca, CaBasal, ceiling, floor).
"""
import ctypes as C

import numpy as np

from . import _native
from .abi import (FIELDS, HS_KIND_CHAN, HS_KIND_CHAN2D, HS_KIND_COMPT, HS_KIND_POOL,
                  HS_KIND_SYNCHAN, HS_PREC_FP64, CellModel)


class _Zombie:
    _kind = None

    def __init__(self, solver, index):
        object.__setattr__(self, "_s", solver)
        object.__setattr__(self, "_i", int(index))

    def __getattr__(self, name):
        if name not in FIELDS:
            raise AttributeError(name)
        return self._s._get(self._kind, FIELDS[name], self._i)

    def __setattr__(self, name, value):
        if name not in FIELDS:
            raise AttributeError(name)
        self._s._set(self._kind, FIELDS[name], self._i, value)


class Compartment(_Zombie):
    _kind = HS_KIND_COMPT


class HHChannel(_Zombie):
    _kind = HS_KIND_CHAN


class CaConc(_Zombie):
    _kind = HS_KIND_POOL

    def setTauB(self, tau, B):
        _native.check(_native.load().hs_set_tau_b(self._s._h, self._i, tau, B))


class HHChannel2D(_Zombie):
    _kind = HS_KIND_CHAN2D


class SynChan(_Zombie):
    _kind = HS_KIND_SYNCHAN

    def add_spike(self, time, weight=1.0, delay=0.0):
        """`Synapse::addSpike` on a synapse of this SynChan's handler: the
        event is queued for time + delay with the synapse's weight."""
        self._s.push_events([self._i], [float(time) + float(delay)], [weight])


class HSolve:
    """One HSolve instance on the GPU (FP64, reference operation order)."""

    def __init__(self, model: CellModel, dt=50e-6):
        self.model = model
        self._dt = float(dt)
        self._ca_advance = 1
        self._h = None
        self._desc = None
        self._path = None
        self._grid_user = dict(vMin=-0.1, vMax=0.05, vDiv=3000, caMin=0.0, caMax=1.0, caDiv=3000)

    # -- fields ------------------------------------------------------------
    @property
    def dt(self):
        return self._dt

    @dt.setter
    def dt(self, v):
        if v < 0.0:
            raise ValueError("HSolve: 'dt' must be positive")
        self._dt = float(v)

    @property
    def caAdvance(self):
        return self._ca_advance

    @caAdvance.setter
    def caAdvance(self, v):
        if v not in (0, 1):
            raise ValueError("HSolve: caAdvance should be either 0 or 1")
        self._ca_advance = int(v)
        if self._h:
            _native.check(_native.load().hs_set_ca_advance(self._h, self._ca_advance))

    @property
    def target(self):
        return self._path

    @target.setter
    def target(self, seed):
        """Seed compartment index (the compartment found under the path)."""
        if self._dt == 0.0:
            raise ValueError("HSolve::setPath(): Must set 'dt' first.")
        self._setup(int(seed))
        self._path = int(seed)

    def _grid(self):
        vmin, vmax, camin, camax = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        vdiv, cadiv = C.c_int(), C.c_int()
        _native.check(_native.load().hs_get_table_grid(self._h, C.byref(vmin), C.byref(vmax), C.byref(vdiv),
                                                       C.byref(camin), C.byref(camax), C.byref(cadiv)))
        return dict(vMin=vmin.value, vMax=vmax.value, vDiv=vdiv.value,
                    caMin=camin.value, caMax=camax.value, caDiv=cadiv.value)

    def __getattr__(self, name):
        if name in ("vMin", "vMax", "vDiv", "caMin", "caMax", "caDiv"):
            if self.__dict__.get("_h"):
                return self._grid()[name]
            return self.__dict__["_grid_user"][name]
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in ("vMin", "vMax", "vDiv", "caMin", "caMax", "caDiv"):
            self._grid_user[name] = value
            return
        object.__setattr__(self, name, value)

    # -- lifecycle -----------------------------------------------------------
    def _setup(self, seed):
        L = _native.load()
        if self._h:
            L.hs_destroy(self._h)
            self._h = None
        self._desc = self.model.desc()
        h = C.c_void_p()
        _native.check(L.hs_create(C.byref(self._desc), seed, self._dt, HS_PREC_FP64, C.byref(h)))
        self._h = h
        _native.check(L.hs_set_ca_advance(self._h, self._ca_advance))

    def reinit(self, clock_dt=None):
        """HSolve::reinit: dt_ becomes the clock dt."""
        clock_dt = self._dt if clock_dt is None else float(clock_dt)
        _native.check(_native.load().hs_reinit(self._h, clock_dt))
        self._dt = clock_dt

    def process(self, nsteps=1):
        _native.check(_native.load().hs_process(self._h, int(nsteps)))

    @property
    def cluster_ctas(self):
        """CTAs stepping the cell (hs_get_cluster_ctas); set 0 for the size
        rule, 1 for one CTA, 2..8 for a thread-block cluster."""
        out = C.c_uint32()
        _native.check(_native.load().hs_get_cluster_ctas(self._h, C.byref(out)))
        return out.value

    @cluster_ctas.setter
    def cluster_ctas(self, v):
        _native.check(_native.load().hs_set_cluster_ctas(self._h, int(v)))

    def sync(self):
        _native.check(_native.load().hs_sync(self._h))

    def close(self):
        if self.__dict__.get("_h"):
            _native.load().hs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- access ---------------------------------------------------------------
    def _get(self, kind, field, index):
        out = C.c_double()
        _native.check(_native.load().hs_get_field(self._h, kind, field, index, C.byref(out)))
        return out.value

    def _set(self, kind, field, index, value):
        _native.check(_native.load().hs_set_field(self._h, kind, field, index, float(value)))

    def compartment(self, i):
        return Compartment(self, i)

    def channel(self, i):
        return HHChannel(self, i)

    def pool(self, i):
        return CaConc(self, i)

    def chan2d(self, i):
        return HHChannel2D(self, i)

    def synchan(self, i):
        return SynChan(self, i)

    def vm(self):
        out = np.empty(self.model.n_compt)
        _native.check(_native.load().hs_read_vm(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), len(out)))
        return out

    def ca(self):
        out = np.empty(len(self.model.pool_compt))
        if len(out):
            _native.check(_native.load().hs_read_ca(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), len(out)))
        return out

    def dif(self):
        """C of each DifShell, bFree of each DifBuffer (0 for an MMPump), in
        the description's order."""
        out = np.empty(len(self.model.dif_kind))
        if len(out):
            _native.check(_native.load().hs_read_dif(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), len(out)))
        return out

    def record(self, compts, stride, capacity):
        a = np.ascontiguousarray(compts, np.uint32)
        _native.check(_native.load().hs_record(self._h, a.ctypes.data_as(C.POINTER(C.c_uint32)), len(a),
                                               int(stride), int(capacity)))
        self._rec = (a, int(capacity))

    def record_values(self, entries, stride, capacity):
        """Record, every `stride` steps on the device, the values the solver
        sends to objects it does not own: entries are (kind, field, index)
        with (HS_KIND_COMPT, Vm), (HS_KIND_CHAN, Ik or Gk), (HS_KIND_POOL,
        Ca); fields by name or code.  Read with trace()."""
        from .abi import FIELDS
        kinds = np.ascontiguousarray([e[0] for e in entries], np.int32)
        fields = np.ascontiguousarray([FIELDS[e[1]] if isinstance(e[1], str) else e[1] for e in entries], np.int32)
        index = np.ascontiguousarray([e[2] for e in entries], np.uint32)
        pi = C.POINTER(C.c_int)
        _native.check(_native.load().hs_record_values(self._h, kinds.ctypes.data_as(pi), fields.ctypes.data_as(pi),
                                                      index.ctypes.data_as(C.POINTER(C.c_uint32)), len(index),
                                                      int(stride), int(capacity)))
        self._rec = (index, int(capacity))

    def trace(self):
        a, cap = self._rec
        out = np.empty((cap, len(a)))
        n = C.c_uint32()
        _native.check(_native.load().hs_read_trace(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), cap,
                                                   C.byref(n)))
        return out[:min(n.value, cap)].T

    def spikes(self):
        n = C.c_uint32()
        L = _native.load()
        _native.check(L.hs_read_spikes(self._h, None, None, 0, C.byref(n)))
        g = np.empty(n.value, np.uint32)
        t = np.empty(n.value)
        _native.check(L.hs_read_spikes(self._h, g.ctypes.data_as(C.POINTER(C.c_uint32)),
                                       t.ctypes.data_as(C.POINTER(C.c_double)), n.value, C.byref(n)))
        return g, t

    def add_inject(self, compt, value):
        _native.check(_native.load().hs_add_inject(self._h, compt, value))

    def add_gkek(self, compt, gk, ek):
        _native.check(_native.load().hs_add_gkek(self._h, compt, gk, ek))

    def add_conc(self, chan, conc):
        """The `concen` message of a zombie HHChannel (HSolve::addConc): the
        external concentration its Ca-dependent gate reads."""
        _native.check(_native.load().hs_add_conc(self._h, chan, conc))

    def add_ica(self, pool, ica):
        """The `current` message of a zombie CaConc (HSolve::iCa)."""
        _native.check(_native.load().hs_add_ica(self._h, pool, ica))

    def push_events(self, syn, time, weight):
        """Queue synaptic events at run time (SimpleSynHandler::addSpike):
        event e reaches SynChan syn[e] at time[e] (spike time + synapse
        delay) with weight[e]; delivered by the next process()."""
        syn = np.ascontiguousarray(np.atleast_1d(syn), dtype=np.uint32)
        time = np.ascontiguousarray(np.atleast_1d(time), dtype=np.float64)
        weight = np.ascontiguousarray(np.atleast_1d(weight), dtype=np.float64)
        if not (len(syn) == len(time) == len(weight)):
            raise ValueError("syn, time and weight differ in length")
        _native.check(_native.load().hs_push_events(
            self._h, syn.ctypes.data_as(C.POINTER(C.c_uint32)),
            time.ctypes.data_as(C.POINTER(C.c_double)),
            weight.ctypes.data_as(C.POINTER(C.c_double)), len(syn)))


def _handles(solvers):
    hs = [s._h for s in solvers]
    if any(h is None for h in hs):
        raise ValueError("every HSolve needs its target set")
    return hs


def process_group(solvers, nsteps):
    """hs_process(s, nsteps) for every HSolve in `solvers`, in one launch
    per cluster size (hs_process_group): bit-identical to stepping each
    alone."""
    hs = _handles(solvers)
    arr = (C.c_void_p * len(hs))(*[h.value for h in hs])
    _native.check(_native.load().hs_process_group(arr, len(hs), int(nsteps)))


class Tick:
    """The HSolves of one clock tick (the Clock processes a tick's objects
    in turn, scheduling/Clock.cpp:872-921), stepped together by
    hs_process_group.  For a loop of short calls: the handle array is built
    once and again only when a member's solver changed (a new target)."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        self._hs = None
        self._arr = None

    def process(self, nsteps=1):
        hs = [s._h for s in self.solvers]
        if self._hs is None or any(a is not b for a, b in zip(hs, self._hs)):
            hs = _handles(self.solvers)
            self._arr = (C.c_void_p * len(hs))(*[h.value for h in hs])
            self._hs = hs
        _native.check(_native.load().hs_process_group(self._arr, len(hs), int(nsteps)))
