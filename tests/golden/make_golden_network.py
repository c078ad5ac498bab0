#!/usr/bin/env python3
"""Three cells coupled by spikes under the REFERENCE, each with its own
HSolve, for moose_gb300.network.

Branched HH cells with two SynChans each (models.active_cell without the
K(Ca) channel, so that no libm call is on the path, and without queued
events), built in the reference pymoose by make_golden_active.build_moose
under /net0 .. /net2; cell 0 gets a soma inject.  Each cell's SpikeGen
drives synapses of other cells through ``spikeOut`` -> ``addSpike`` with
delays of 1.5 to 3.1 ms (a ring plus a feed-forward link).  0.15 s at
25 us; a Table per cell records the soma Vm every step and one per
SpikeGen its spike times.

Output: ``tests/golden/network_golden.npz`` (the three models, the
connections, the traces and spikes).  Prerequisite: the reference build
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

DT, NSTEPS = 25e-6, 6000
# (source cell, its SpikeGen, target cell, its SynChan, delay, weight)
CONNECTIONS = [(0, 0, 1, 0, 1.5e-3, 1.0), (1, 0, 2, 1, 2.0e-3, 1.0), (2, 0, 0, 1, 3.1e-3, 0.7),
               (0, 0, 2, 0, 1.75e-3, 1.3)]


def network_models():
    out = []
    for i in range(3):
        rng = np.random.default_rng([71, i])
        parent, d, L = models.branched_morphology(rng, 30 + 10 * i, 0.5, 3)
        m = models.active_cell(parent, d, L, inject=0.6e-9 if i == 0 else 0.0, n_syn=2, rng=rng, t_end=0.15,
                               gca=10.0, gkca=0.0)
        for k in list(vars(m)):
            if k.startswith("c2d_"):
                setattr(m, k, getattr(m, k)[:0])
        m.gates2d = []
        for k in ("ev_syn", "ev_time", "ev_weight"):
            setattr(m, k, getattr(m, k)[:0])
        m.syn_Gbar = np.full(len(m.syn_compt), 2e-8)
        out.append(m)
    return out


def main():
    import moose
    ms = network_models()
    built = [build_moose(m, DT, cell="/net%d" % i, library="/lib%d" % i) for i, m in enumerate(ms)]
    for t in range(9):
        moose.setClock(t, DT)
    for src, gen, dst, syn, delay, weight in CONNECTIONS:
        s = synapse(built[dst][3][syn], 0)
        s.delay, s.weight = delay, weight
        moose.connect(built[src][4][gen], "spikeOut", s, "addSpike")
    vt, st = [], []
    for i, (comp, pools, chans, handlers, gens) in enumerate(built):
        t = moose.Table("/net%d/vm" % i)
        moose.connect(t, "requestOut", comp[0], "getVm")
        vt.append(t)
        s = moose.Table("/net%d/spk" % i)
        moose.connect(gens[0], "spikeOut", s, "input")
        st.append(s)
        h = moose.HSolve("/net%d/hsolve" % i)
        h.dt = DT
        h.target = comp[ms[i].seed].path
    moose.reinit()
    moose.start(NSTEPS * DT)
    out = {"dt": DT, "nsteps": NSTEPS, "connections": np.array(CONNECTIONS)}
    for i, m in enumerate(ms):
        out["vm%d" % i] = np.array(vt[i].vector)
        out["spikes%d" % i] = np.array(st[i].vector)
        out.update(save_model(m, prefix="m%d_" % i))
    np.savez_compressed(os.path.join(HERE, "network_golden.npz"), **out)
    print("network: spikes per cell", [len(s.vector) for s in st])


if __name__ == "__main__":
    main()
