#!/usr/bin/env python3
"""Stats and SpikeStats under the REFERENCE HSolve, for moose_gb300.stats.

A 41-compartment HH cable (models.config1_cell) with a constant soma
inject, built in the reference pymoose by make_golden_active.build_moose,
solved by the reference HSolve for 0.2 s at 25 us.  A ``SpikeStats``
(tick 7, every 40 steps, a window of 25) takes the soma SpikeGen's
``spikeOut``; a ``Stats`` (tick 17, every 20 steps, a window of 30)
requests the soma's Vm through the zombie getter.  Saved: both objects'
fields after the run, the SpikeGen's spike times (a Table on spikeOut), the
run's sizes and the model (``save_model``).

Output: ``tests/golden/stats_golden.npz``.  Prerequisite: the reference
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

DT, NSTEPS = 25e-6, 8000
SS_STRIDE, SS_WINDOW = 40, 25
ST_STRIDE, ST_WINDOW = 20, 30
FIELDS = ("mean", "sdev", "sum", "num", "wmean", "wsdev", "wsum", "wnum")


def stats_model():
    m = models.config1_cell(n_cable=40, inject=0.0)
    m.inject[:] = 0.0
    m.inject[0] = 0.35e-9
    for k in ("stim_compt", "stim_step", "stim_value"):
        setattr(m, k, getattr(m, k)[:0])
    return m


def main():
    import moose
    m = stats_model()
    comp, pools, chans, handlers, gens = build_moose(m, DT)
    for t in range(8):
        moose.setClock(t, DT)
    moose.setClock(7, DT * SS_STRIDE)
    moose.setClock(17, DT * ST_STRIDE)
    ss = moose.SpikeStats("/cell/sstats")
    ss.windowLength = SS_WINDOW
    moose.connect(gens[0], "spikeOut", ss, "addSpike")
    st = moose.Stats("/cell/vstats")
    st.windowLength = ST_WINDOW
    moose.connect(st, "requestOut", comp[0], "getVm")
    spk = moose.Table("/cell/spk")
    moose.connect(gens[0], "spikeOut", spk, "input")
    h = moose.HSolve("/cell/hsolve")
    h.dt = DT
    h.target = comp[m.seed].path
    moose.reinit()
    moose.start(NSTEPS * DT)
    out = {"dt": DT, "nsteps": NSTEPS, "ss_stride": SS_STRIDE, "ss_window": SS_WINDOW,
           "st_stride": ST_STRIDE, "st_window": ST_WINDOW, "spikes": np.array(spk.vector)}
    for f in FIELDS:
        out["ss_" + f] = np.array(getattr(ss, f))
        out["st_" + f] = np.array(getattr(st, f))
    np.savez_compressed(os.path.join(HERE, "stats_golden.npz"), **out, **save_model(m))
    print("stats: %d spikes, SpikeStats mean %g, Stats mean %g" % (len(spk.vector), ss.mean, st.mean))


if __name__ == "__main__":
    main()
