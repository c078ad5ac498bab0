#!/usr/bin/env python3
"""SynChans driven by TimeTables under the REFERENCE HSolve, for
moose_gb300.inputs.

A branched 60-compartment HH cell with six SynChans (models.active_cell,
without the K(Ca) channel so that no libm call is on the path), built in
the reference pymoose by make_golden_active.build_moose; each SynChan's
synapse is driven by a ``TimeTable`` on tick 8 (every 4 steps of 25 us):
tables with entries closer together than a tick (sent one per tick, so
they lag), entries between steps, synapse delays of 0 to 2.5 ms and
different weights; one table on tick 0 instead (it runs every step there,
before the handler, so its entries can reach the synapse in the step
they are sent in).  A Table on tick 8 records the soma Vm; 0.1 s.

Output: ``tests/golden/timetable_golden.npz`` (the model, each table's
entries, delay and weight, the trace).  Prerequisite: the reference build
(``python oracle/build_ref.py``).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
sys.path.insert(0, os.path.join(REPO, "moose-core_gb300"))

from make_golden_active import build_moose, save_model, synapse  # noqa: E402
from moose_gb300 import models  # noqa: E402

DT, NSTEPS, STRIDE = 25e-6, 4000, 4
EARLY = (3,)      # these SynChans' tables run on tick 0, before the handler


def timetable_model():
    rng = np.random.default_rng(61)
    parent, d, L = models.branched_morphology(rng, 60, 0.5, 3)
    m = models.active_cell(parent, d, L, inject=0.1e-9, n_syn=6, rng=rng, t_end=0.1, gca=10.0, gkca=0.0)
    for k in list(vars(m)):
        if k.startswith("c2d_"):
            setattr(m, k, getattr(m, k)[:0])
    m.gates2d = []
    for k in ("ev_syn", "ev_time", "ev_weight"):
        setattr(m, k, getattr(m, k)[:0])
    m.syn_Gbar = m.syn_Gbar * 20.0
    return m


def tables():
    """Per SynChan: entries, synapse delay, weight."""
    rng = np.random.default_rng(62)
    out = {}
    for k in range(6):
        base = np.sort(rng.uniform(0.002, 0.09, 8))
        if k % 2 == 0:                        # bursts closer than one tick (0.1 ms)
            base = np.sort(np.concatenate([base, base[:3] + 3e-5, base[:2] + 6.1e-5]))
        out[k] = (base, [0.0, 1e-3, 2.5e-3, 0.0, 3.7e-4, 1.25e-5][k], [1.0, 0.5, 2.0, 1.5, 0.8, 1.2][k])
    return out


def main():
    import moose
    m = timetable_model()
    comp, pools, chans, handlers, gens = build_moose(m, DT)
    for t in range(8):
        moose.setClock(t, DT)
    moose.setClock(8, DT * STRIDE)
    tt = tables()
    for k, (times, delay, weight) in tt.items():
        s = synapse(handlers[k], 0)
        s.delay, s.weight = delay, weight
        t = moose.TimeTable("/cell/tt%d" % k)
        t.vector = times
        moose.connect(t, "eventOut", s, "addSpike")
        if k in EARLY:
            moose.useClock(0, t.path, "process")
    vt = moose.Table("/cell/vm")
    moose.connect(vt, "requestOut", comp[0], "getVm")
    h = moose.HSolve("/cell/hsolve")
    h.dt = DT
    h.target = comp[m.seed].path
    moose.reinit()
    moose.start(NSTEPS * DT)
    out = {"dt": DT, "nsteps": NSTEPS, "stride": STRIDE, "vm": np.array(vt.vector),
           "final_vm": np.array([c.Vm for c in comp])}
    for k, (times, delay, weight) in tt.items():
        out["tt%d_times" % k] = times
        out["tt%d_delay" % k] = np.array(delay)
        out["tt%d_weight" % k] = np.array(weight)
    np.savez_compressed(os.path.join(HERE, "timetable_golden.npz"), **out, **save_model(m))
    print("timetable: %d samples, soma Vm range %.4f..%.4f" % (len(vt.vector), min(vt.vector), max(vt.vector)))


if __name__ == "__main__":
    main()
