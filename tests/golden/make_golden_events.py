#!/usr/bin/env python3
"""Golden traces for synaptic events queued at run time, from the REFERENCE
``moose`` module with an HSolve.

The cell: the seeded 60-compartment branched tree of ``active_branched_kca``
(HH Na/K, Ca(HVA) feeding a CaConc in every compartment, a SpikeGen on the
soma) without its HHChannel2D, so that no libm call is on the solver's path,
and 12 SynChans.  Each SynChan's SimpleSynHandler has two synapses: synapse 0
with delay 0 and the SynChan's weight, synapse 1 with its own weight and a
delay of 0.4-2.5 ms.  Events reach the handlers three ways
(``synapse/Synapse.cpp:104-113`` -> ``synapse/SimpleSynHandler.cpp:86-90``):
  * ``Synapse::addSpike`` before ``moose.reinit()``: dropped by
    ``SimpleSynHandler::vReinit``;
  * the model's Poisson trains, queued on synapse 0 right after reinit (as
    the description's events of every other golden);
  * ``Synapse::addSpike`` between ``moose.start`` chunks (every CHUNK steps),
    on either synapse, with spike times from 1 ms in the past (delivered at
    the next step) to 8 ms ahead, and some on synapse 0 exactly at a future
    step's clock time ``dt * step`` (delivered at that step:
    ``time <= currTime``, ``scheduling/Clock.cpp:729``).
Saved with the model: the pushes (chunk step, SynChan, synapse, spike time),
the synapses' weights and delays, Vm samples every STRIDE steps, the final
Vm and the SpikeGen's spike times.  Output: ``tests/golden/active_events.npz``.
Prerequisite: the reference build (``python oracle/build_ref.py``).
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

DT, NSTEPS, STRIDE, CHUNK = 25e-6, 4000, 4, 200
N_SYN = 12


def event_cell():
    rng = np.random.default_rng(7)
    parent, d, L = models.branched_morphology(rng, 60, 0.5, 4)
    m = models.active_cell(parent, d, L, inject=0.4e-9, n_syn=N_SYN, syn_rate=40.0, t_end=0.1,
                           rng=rng, gca=20.0, gkca=0.0, inject_step=400)
    for k in list(vars(m)):
        if k.startswith("c2d_"):
            setattr(m, k, getattr(m, k)[:0])
    m.gates2d = []
    m.seed = 0
    return m


def synapses(m, rng):
    """weight[k, j], delay[k, j] of synapse j of SynChan k."""
    w = np.empty((N_SYN, 2))
    dl = np.zeros((N_SYN, 2))
    for k in range(N_SYN):
        ev = m.ev_weight[m.ev_syn == k]
        w[k, 0] = ev[0] if len(ev) else 0.5e-9
    w[:, 1] = np.exp(rng.normal(np.log(0.8e-9), 0.4, N_SYN))
    dl[:, 1] = rng.uniform(0.4e-3, 2.5e-3, N_SYN)
    return w, dl


def pushes(rng):
    """(step, syn, synapse, spike time) rows: pushed once `step` steps ran."""
    rows = []
    for step in range(CHUNK, NSTEPS, CHUNK):
        t0 = DT * step
        for k in range(N_SYN):
            n = rng.poisson(150.0 * 9e-3)
            for t in np.sort(rng.uniform(t0 - 1e-3, t0 + 8e-3, n)):
                rows.append((step, k, int(rng.integers(0, 2)), float(t)))
        # on a future step's clock time exactly (synapse 0: no delay)
        for q in (1, 7, 60):
            k = int(rng.integers(0, N_SYN))
            rows.append((step, k, 0, DT * (step + q)))
    return np.array([r[0] for r in rows], np.int64), np.array([r[1] for r in rows], np.int64), \
        np.array([r[2] for r in rows], np.int64), np.array([r[3] for r in rows])


def make():
    import moose
    m = event_cell()
    rng = np.random.default_rng(11)
    w, dl = synapses(m, rng)
    p_step, p_syn, p_sy, p_time = pushes(rng)
    pre_syn = rng.integers(0, N_SYN, 20)
    pre_time = rng.uniform(0.0, DT * NSTEPS, 20)

    comp, pools, chans, handlers, gens = build_moose(m, DT)
    for k, sh in enumerate(handlers):
        sh.numSynapses = 2
        for j in range(2):
            synapse(sh, j).weight = float(w[k, j])
            synapse(sh, j).delay = float(dl[k, j])
    for t in range(8):
        moose.setClock(t, DT)
    moose.setClock(8, DT * STRIDE)
    tabs = []
    rec = list(range(0, 60, 6))
    for i in rec:
        t = moose.Table("/cell/vm%d" % i)
        moose.connect(t, "requestOut", comp[i], "getVm")
        tabs.append(t)
    spk = moose.Table("/cell/spk")
    moose.connect(gens[0], "spikeOut", spk, "input")
    h = moose.HSolve("/cell/hsolve")
    h.dt = DT
    h.target = comp[m.seed].path
    for k, t in zip(pre_syn, pre_time):
        synapse(handlers[int(k)], 1).addSpike(float(t))
    moose.reinit()
    for e in range(len(m.ev_syn)):
        synapse(handlers[int(m.ev_syn[e])], 0).addSpike(float(m.ev_time[e]))
    stops = sorted(set(m.stim_step.tolist()) | set(p_step.tolist()) | {NSTEPS})
    cur = 0
    for step in stops:
        if step > cur:
            moose.start((step - cur) * DT)
            cur = step
        for i in np.nonzero(m.stim_step == step)[0]:
            comp[int(m.stim_compt[i])].inject = float(m.stim_value[i])
        for i in np.nonzero(p_step == step)[0]:
            synapse(handlers[int(p_syn[i])], int(p_sy[i])).addSpike(float(p_time[i]))
    vm = np.array([t.vector for t in tabs])
    out = dict(dt=DT, nsteps=NSTEPS, stride=STRIDE, chunk=CHUNK, rec=np.array(rec), vm=vm,
               final_vm=np.array([c.Vm for c in comp]), spikes=np.array(spk.vector),
               syn_weight=w, syn_delay=dl, push_step=p_step, push_syn=p_syn,
               push_synapse=p_sy, push_time=p_time, pre_syn=pre_syn, pre_time=pre_time,
               **save_model(m))
    np.savez_compressed(os.path.join(HERE, "active_events.npz"), **out)
    print("events: %d pushed in %d chunks, %d queued at reinit, %d dropped by reinit; "
          "samples %s, spikes %d" % (len(p_time), len(set(p_step.tolist())), len(m.ev_syn),
                                     len(pre_time), vm.shape, len(spk.vector)))


if __name__ == "__main__":
    make()
