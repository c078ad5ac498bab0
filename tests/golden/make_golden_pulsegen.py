#!/usr/bin/env python3
"""PulseGens driving compartments under the REFERENCE HSolve, for
moose_gb300.inputs.add_pulsegen.

A 41-compartment HH cable (models.config1_cell) built in the reference
pymoose by make_golden_active.build_moose, one compartment with its own
inject field.  Two free-running PulseGens send ``output`` to
``injectMsg``: one into the soma on tick 0 (two pulses, a non-zero base
level, which PulseGen::reinit also sends), one into the compartment with
the inject field on tick 2 at three steps per tick (its output reaches
only the steps its tick fires on); a third, on tick 9 after the solver,
reaches each step after the one its tick fires on.  Two StimulusTables on tick 0 send
``output`` to ``injectMsg`` of two more compartments: one read at the
clock time and looping, one advancing by its own step size.  Tables
record the PulseGens' compartments' Vm; 0.06 s at 25 us.

Output: ``tests/golden/pulsegen_golden.npz``.  Prerequisite: the reference
build (``python oracle/build_ref.py``).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
sys.path.insert(0, os.path.join(REPO, "moose-core_gb300"))

from make_golden_active import build_moose, save_model  # noqa: E402
from moose_gb300 import models  # noqa: E402

DT, NSTEPS = 25e-6, 2400
PULSES = {
    # compartment: (level, width, delay, baseLevel, tick, steps per tick)
    0: ([4e-10, 7e-10], [0.01, 0.005], [0.005, 0.02], 5e-11, 0, 1),
    3: ([3e-10], [0.003], [0.002], 0.0, 2, 3),
    # on tick 9, after the solver: its output reaches the next step
    20: ([5e-10, 2e-10], [0.004, 0.006], [0.008, 0.01], 2e-11, 9, 2),
}
FIELD_INJECT = {3: 2e-11}
STIMTABLES = {
    # compartment: (vector, startTime, stopTime, stepSize, doLoop, loopTime)
    7: ([0.0, 3e-10, -1e-10, 2e-10, 0.0], 0.004, 0.024, 0.0, True, 0.03),
    12: ([1e-10, 4e-10, 0.0], 0.01, 0.04, 1.3 * 25e-6, False, 0.0),
}


def pulse_model():
    m = models.config1_cell(n_cable=40, inject=0.0)
    m.inject[:] = 0.0
    for c, v in FIELD_INJECT.items():
        m.inject[c] = v
    for k in ("stim_compt", "stim_step", "stim_value"):
        setattr(m, k, getattr(m, k)[:0])
    return m


def main():
    import moose
    m = pulse_model()
    comp, pools, chans, handlers, gens = build_moose(m, DT)
    for t in range(8):
        moose.setClock(t, DT)
    for c, (level, width, delay, base, tick, k) in PULSES.items():
        pg = moose.PulseGen("/cell/pg%d" % c)
        pg.count = len(level)
        for i in range(len(level)):
            pg.level[i], pg.width[i], pg.delay[i] = level[i], width[i], delay[i]
        pg.baseLevel = base
        pg.trigMode = 0
        moose.connect(pg, "output", comp[c], "injectMsg")
        if tick != 0:
            moose.setClock(tick, DT * k)
            moose.useClock(tick, pg.path, "process")
    for c, (vec, start, stop, step, loop, loop_t) in STIMTABLES.items():
        st = moose.StimulusTable("/cell/st%d" % c)
        st.vector = vec
        st.startTime, st.stopTime, st.stepSize = start, stop, step
        st.doLoop, st.loopTime = loop, loop_t
        moose.connect(st, "output", comp[c], "injectMsg")
    tabs = []
    for c in PULSES:
        t = moose.Table("/cell/vm%d" % c)
        moose.connect(t, "requestOut", comp[c], "getVm")
        tabs.append(t)
    h = moose.HSolve("/cell/hsolve")
    h.dt = DT
    h.target = comp[m.seed].path
    moose.reinit()
    moose.start(NSTEPS * DT)
    out = {"dt": DT, "nsteps": NSTEPS, "vm": np.array([t.vector for t in tabs]),
           "final_vm": np.array([c.Vm for c in comp]), "rec": np.array(list(PULSES))}
    np.savez_compressed(os.path.join(HERE, "pulsegen_golden.npz"), **out, **save_model(m))
    print("pulsegen: %d samples; soma Vm max %.4f" % (tabs[0].vector.size, max(tabs[0].vector)))


if __name__ == "__main__":
    main()
