"""Batched HSolve: many cells stepped by one persistent kernel.

Each cell is set up exactly like the drop-in ``HSolve`` (same Hines setup,
same reinit semantics).  ``precision=HS_PREC_FP64`` keeps the drop-in's exact
arithmetic (bit-identical results); ``HS_PREC_MIXED`` runs gates, tables,
synapses and Ca pools in FP32 with an FP64 matrix and solve.
"""
import ctypes as C

import numpy as np

from . import _native
from .abi import HS_PREC_FP64, HsBatchTuning, HsCellDesc


class Batch:
    def __init__(self, cells, dt, precision=HS_PREC_FP64, seeds=None, threads_per_cta=0,
                 ctas_per_sm=0, steps_per_launch=0, use_graph=True, forest_nodes=0, max_ctas=0, elim_warps=0,
                 wait_rounds=0, cluster_ctas=0):
        self.cells = list(cells)
        self.n = len(self.cells)
        descs = (HsCellDesc * self.n)()
        for i, m in enumerate(self.cells):
            descs[i] = m.desc()
        self._descs = descs
        seeds = np.ascontiguousarray([m.seed for m in self.cells] if seeds is None else seeds, np.uint32)
        self._seeds = seeds
        tun = HsBatchTuning(threads_per_cta, ctas_per_sm, steps_per_launch, 1 if use_graph else 0, forest_nodes,
                            max_ctas, elim_warps, wait_rounds, cluster_ctas)
        h = C.c_void_p()
        _native.check(_native.load().hs_batch_create(descs, seeds.ctypes.data_as(C.POINTER(C.c_uint32)), self.n,
                                                     float(dt), int(precision), C.byref(tun), C.byref(h)))
        self._h = h
        self.precision = precision
        self._rec = None

    def close(self):
        if getattr(self, "_h", None):
            _native.load().hs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tune(self, threads_per_cta=0, ctas_per_sm=0, steps_per_launch=0, use_graph=True, forest_nodes=0,
             max_ctas=0, elim_warps=0, wait_rounds=0, cluster_ctas=0):
        """New launch shape.  On a mixed batch a new ctas_per_sm or
        forest_nodes rebuilds the layout: reinit (and re-register recording
        and inject targets) before the next process()."""
        t = HsBatchTuning(threads_per_cta, ctas_per_sm, steps_per_launch, 1 if use_graph else 0, forest_nodes,
                          max_ctas, elim_warps, wait_rounds, cluster_ctas)
        _native.check(_native.load().hs_batch_tune(self._h, C.byref(t)))

    def reinit(self, dt):
        _native.check(_native.load().hs_batch_reinit(self._h, float(dt)))

    def process(self, nsteps):
        _native.check(_native.load().hs_batch_process(self._h, int(nsteps)))

    def idle(self):
        """True when all queued work has finished (does not wait)."""
        v = C.c_int()
        _native.check(_native.load().hs_batch_idle(self._h, C.byref(v)))
        return bool(v.value)

    def sync(self):
        _native.check(_native.load().hs_batch_sync(self._h))

    def vm(self, cell):
        out = np.empty(self.cells[cell].n_compt)
        _native.check(_native.load().hs_batch_read_vm(self._h, cell, out.ctypes.data_as(C.POINTER(C.c_double)),
                                                      len(out)))
        return out

    def ca(self, cell):
        out = np.empty(len(self.cells[cell].pool_compt))
        if len(out):
            _native.check(_native.load().hs_batch_read_ca(self._h, cell,
                                                          out.ctypes.data_as(C.POINTER(C.c_double)), len(out)))
        return out

    def read_all(self, field="Vm", out=None):
        """Vm (or Ca, field="Ca") of every compartment (pool) of every cell,
        cell after cell in model order, with one device gather and one copy."""
        from .abi import FIELDS
        if field not in ("Vm", "Ca"):
            raise ValueError("field must be 'Vm' or 'Ca'")
        fid = FIELDS[field]
        n = sum(m.n_compt for m in self.cells) if field == "Vm" else sum(len(m.pool_compt) for m in self.cells)
        if out is None:
            out = np.empty(n)
        _native.check(_native.load().hs_batch_read_all(self._h, fid, out.ctypes.data_as(C.POINTER(C.c_double)), n))
        return out

    def record(self, cells, compts, stride, capacity):
        c = np.ascontiguousarray(cells, np.uint32)
        m = np.ascontiguousarray(compts, np.uint32)
        pu = C.POINTER(C.c_uint32)
        _native.check(_native.load().hs_batch_record(self._h, c.ctypes.data_as(pu), m.ctypes.data_as(pu), len(c),
                                                     int(stride), int(capacity)))
        self._rec = (c, m, int(capacity))

    def trace(self):
        """Samples x recorded columns, columns grouped by cell in cell order."""
        c, m, cap = self._rec
        out = np.empty((cap, len(c)))
        n = C.c_uint32()
        _native.check(_native.load().hs_batch_read_trace(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), cap,
                                                         C.byref(n)))
        order = sorted(range(len(c)), key=lambda k: (int(c[k]), k))
        return out[:min(n.value, cap)], [(int(c[k]), int(m[k])) for k in order]

    def trace_window(self, first, count, out=None):
        """Samples [first, first+count) into `out` (a host buffer, e.g. pinned)."""
        ncol = len(self._rec[0])
        if out is None:
            out = np.empty((count, ncol))
        ptr = out.data_ptr() if hasattr(out, "data_ptr") else out.ctypes.data
        _native.check(_native.load().hs_batch_read_trace_window(self._h, int(first), int(count), C.c_void_p(ptr)))
        return out

    def inject_targets(self, cells, compts):
        c = np.ascontiguousarray(cells, np.uint32)
        m = np.ascontiguousarray(compts, np.uint32)
        self._inj = (c, m)
        pu = C.POINTER(C.c_uint32)
        _native.check(_native.load().hs_batch_inject_targets(self._h, c.ctypes.data_as(pu), m.ctypes.data_as(pu),
                                                             len(c)))

    def set_inject(self, values):
        """One value per registered target; `values` may be a numpy array or a
        pinned torch tensor (float64)."""
        ptr = values.data_ptr() if hasattr(values, "data_ptr") else values.ctypes.data
        _native.check(_native.load().hs_batch_set_inject(self._h, C.c_void_p(ptr), len(self._inj[0])))

    def set_modulation(self, kind, cells, index, values):
        """modulation of (cells[k], channel index[k]) = values[k]; kind is
        HS_KIND_CHAN (HHChannel; values <= 0 are ignored, as
        HSolve::setHHmodulation does), HS_KIND_CHAN2D or HS_KIND_SYNCHAN."""
        c = np.ascontiguousarray(cells, np.uint32)
        i = np.ascontiguousarray(index, np.uint32)
        v = np.ascontiguousarray(values, np.float64)
        pu = C.POINTER(C.c_uint32)
        _native.check(_native.load().hs_batch_set_modulation(self._h, int(kind), c.ctypes.data_as(pu),
                                                             i.ctypes.data_as(pu),
                                                             v.ctypes.data_as(C.POINTER(C.c_double)), len(v)))

    def set_inject_at(self, cells, compts, values):
        """inject of (cells[k], compts[k]) = values[k], without allocating
        (hs_batch_set_inject_at; at most 32768 writes per call)."""
        c = np.ascontiguousarray(cells, np.uint32)
        m = np.ascontiguousarray(compts, np.uint32)
        v = np.ascontiguousarray(values, np.float64)
        pu = C.POINTER(C.c_uint32)
        _native.check(_native.load().hs_batch_set_inject_at(self._h, c.ctypes.data_as(pu), m.ctypes.data_as(pu),
                                                            v.ctypes.data_as(C.POINTER(C.c_double)), len(v)))

    def push_events(self, cells, syn, time, weight):
        """Queue synaptic events at run time (SimpleSynHandler::addSpike):
        event e reaches SynChan syn[e] of cell cells[e] at time[e] (spike
        time + synapse delay) with weight[e]; delivered from the next
        process(), dropped by reinit()."""
        c = np.ascontiguousarray(np.atleast_1d(cells), np.uint32)
        k = np.ascontiguousarray(np.atleast_1d(syn), np.uint32)
        t = np.ascontiguousarray(np.atleast_1d(time), np.float64)
        w = np.ascontiguousarray(np.atleast_1d(weight), np.float64)
        if not (len(c) == len(k) == len(t) == len(w)):
            raise ValueError("cells, syn, time and weight differ in length")
        pu, pd = C.POINTER(C.c_uint32), C.POINTER(C.c_double)
        _native.check(_native.load().hs_batch_push_events(self._h, c.ctypes.data_as(pu), k.ctypes.data_as(pu),
                                                          t.ctypes.data_as(pd), w.ctypes.data_as(pd), len(t)))

    def spikes(self):
        L = _native.load()
        n = C.c_uint32()
        L.hs_batch_read_spikes(self._h, None, None, None, 0, C.byref(n))
        cells = np.empty(n.value, np.uint32)
        gens = np.empty(n.value, np.uint32)
        t = np.empty(n.value)
        pu = C.POINTER(C.c_uint32)
        _native.check(L.hs_batch_read_spikes(self._h, cells.ctypes.data_as(pu), gens.ctypes.data_as(pu),
                                             t.ctypes.data_as(C.POINTER(C.c_double)), n.value, C.byref(n)))
        return cells, gens, t

    def set_stop_steps(self, stop):
        """Cell c advances only while its step count is below stop[c]
        (None or -1: no limit).  Mixed precision only."""
        a = np.array([np.iinfo(np.uint64).max if (x is None or x < 0) else x for x in stop], np.uint64)
        _native.check(_native.load().hs_batch_set_stop_steps(self._h, a.ctypes.data_as(C.POINTER(C.c_uint64)),
                                                             len(a)))

    def steps(self):
        """dt steps each cell has advanced.  Mixed precision only."""
        out = np.empty(self.n, np.uint64)
        _native.check(_native.load().hs_batch_read_steps(self._h, out.ctypes.data_as(C.POINTER(C.c_uint64)),
                                                         self.n))
        return out

    def spike_counts(self):
        """Spikes recorded so far by each cell.  Mixed precision only."""
        out = np.empty(self.n, np.uint32)
        _native.check(_native.load().hs_batch_read_spike_counts(self._h, out.ctypes.data_as(C.POINTER(C.c_uint32)),
                                                                self.n))
        return out

    def poll(self, first, count):
        """(trace samples [first, first+count), step counts, spike counts) in
        one device round trip.  Mixed precision only."""
        ncol = len(self._rec[0]) if self._rec else 0
        tr = np.empty((count, ncol)) if count else None
        st = np.empty(self.n, np.uint64)
        sc = np.empty(self.n, np.uint32)
        _native.check(_native.load().hs_batch_poll(
            self._h, int(first), int(count), tr.ctypes.data_as(C.POINTER(C.c_double)) if count else None,
            st.ctypes.data_as(C.POINTER(C.c_uint64)), sc.ctypes.data_as(C.POINTER(C.c_uint32))))
        return tr, st, sc

    def device_bytes(self):
        v = C.c_uint64()
        _native.check(_native.load().hs_batch_device_bytes(self._h, C.byref(v)))
        return v.value

    def cell_spikes(self, cell, first=0, capacity=4096):
        """(generator index, time) of the cell's spikes from its `first`-th on,
        and the cell's total spike count.  Mixed precision only."""
        g = np.empty(capacity, np.uint32)
        t = np.empty(capacity)
        n = C.c_uint32()
        _native.check(_native.load().hs_batch_read_cell_spikes(
            self._h, int(cell), int(first), g.ctypes.data_as(C.POINTER(C.c_uint32)),
            t.ctypes.data_as(C.POINTER(C.c_double)), capacity, C.byref(n)))
        k = max(0, min(n.value, capacity + first) - first)
        return g[:k], t[:k], n.value

    def stream(self):
        """The cudaStream_t handle (int) the batch's kernels run on."""
        s = C.c_void_p()
        _native.check(_native.load().hs_batch_stream(self._h, C.byref(s)))
        return s.value or 0

    def info(self):
        nc = C.c_uint64()
        ctas, tpc, spl = C.c_uint32(), C.c_uint32(), C.c_uint32()
        _native.check(_native.load().hs_batch_info(self._h, C.byref(nc), C.byref(ctas), C.byref(tpc), C.byref(spl)))
        nf, ns = C.c_uint32(), C.c_uint32()
        _native.check(_native.load().hs_batch_forests(self._h, C.byref(nf), C.byref(ns)))
        return dict(n_compt=nc.value, n_ctas=ctas.value, threads_per_cta=tpc.value, steps_per_launch=spl.value,
                    n_forests=nf.value, n_shared_forests=ns.value)

    def kernel_time(self):
        """(average ms per stepping launch, launches) since the last call."""
        ms, n = C.c_double(), C.c_uint32()
        _native.check(_native.load().hs_batch_kernel_time(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value
