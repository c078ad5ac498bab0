#!/usr/bin/env python3
"""Golden traces for the solver's message destinations and its Ca-dependent
HHChannel gates, from the REFERENCE ``moose`` module with an HSolve.

The cell: a seeded branched tree (junctions up to 4 children), HH Na/K and
Ca(HVA) feeding a CaConc in every compartment (as the workload cells), and
  * an SK-type channel in every compartment whose Z gate reads its
    compartment's CaConc (``useConcentration``, concOut -> concen: HSolve's
    caDepend path, the Ca table of ``createLookupTables``);
  * in three compartments a second SK-type channel with no pool: its Z gate
    reads the concentration sent to it (HSolve::addConc), the V row while
    that is 0 (``hsolve/HSolveActive.cpp:250-270``).
Three StimulusTables on tick 0 send, every step (after sending 0 at reinit):
  * the soma's ``injectMsg``          -> HSolve::addInject
  * each external SK's ``concen``     -> HSolve::addConc
  * the soma CaConc's ``current``     -> HSolve::iCa
(``hsolve/HSolveInterface.cpp:213-259, 469-480``; zombie forwarding in
``hsolve/ZombieCompartment.cpp:192-195``, ``ZombieHHChannel.cpp:178-182``,
``ZombieCaConc.cpp:128-132``).  Tables record the value each StimulusTable
sent at each step (``Table::input``), Vm and Ca samples every 10 steps and
the final Vm.  Output: ``tests/golden/active_msgs.npz`` (the model is saved
with it).  Prerequisite: the reference build (``python oracle/build_ref.py``).
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
from moose_gb300.abi import CellModel  # noqa: E402

DT, NSTEPS, STRIDE = 25e-6, 2000, 10
EXT_COMPTS = (0, 7, 19)


def sk_tables(cmin=0.0, cmax=0.1, cdivs=500, kd=0.03, tau=5e-3):
    """Z gate of an SK-type channel on concentration: zinf = c^4/(c^4+kd^4),
    tau constant (A = zinf/tau, B = 1/tau)."""
    c = np.linspace(cmin, cmax, cdivs + 1)
    zinf = c ** 4 / (c ** 4 + kd ** 4)
    return (cmin, cmax, zinf / tau, np.full_like(c, 1.0 / tau))


def msg_cell(seed=7, n=40, gsk=20.0):
    rng = np.random.default_rng(seed)
    parent, d, L = models.branched_morphology(rng, n, 0.5, 4)
    m = models.active_cell(parent, d, L, inject=0.0, gca=15.0, gkca=0.0)
    a = {k: getattr(m, k) for k in vars(m) if not k.startswith("_") and isinstance(getattr(m, k), np.ndarray)}
    for k in list(a):
        if k.startswith("c2d_"):
            a[k] = a[k][:0]
    area = m.meta["pool_diameter"] * m.meta["pool_length"] * models.PI
    gates = list(m.gates) + [sk_tables()]
    zg = len(gates) - 1
    # channels: per compartment in message order; SK after the three
    # channels of active_cell, then the external SKs (created last)
    comp = [m.chan_compt, np.arange(n, dtype=np.uint32), np.array(EXT_COMPTS, np.uint32)]
    nsk, nx = n, len(EXT_COMPTS)
    extra = nsk + nx

    def cat(name, v_sk, v_ext):
        return np.concatenate([a[name], np.asarray(v_sk, a[name].dtype), np.asarray(v_ext, a[name].dtype)])

    a["chan_compt"] = np.concatenate(comp)
    a["chan_Gbar"] = cat("chan_Gbar", gsk * area, gsk * area[list(EXT_COMPTS)])
    a["chan_Ek"] = cat("chan_Ek", np.full(nsk, -77e-3), np.full(nx, -77e-3))
    for f, v in (("chan_Xpower", 0.0), ("chan_Ypower", 0.0), ("chan_Zpower", 1.0), ("chan_instant", 0),
                 ("chan_modulation", 1.0), ("chan_use_conc", 1), ("chan_X", 0.0), ("chan_Y", 0.0),
                 ("chan_Z", 0.0), ("chan_ca_target", -1)):
        a[f] = cat(f, np.full(nsk, v), np.full(nx, v))
    a["chan_xgate"] = cat("chan_xgate", np.full(nsk, -1), np.full(nx, -1))
    a["chan_ygate"] = cat("chan_ygate", np.full(nsk, -1), np.full(nx, -1))
    a["chan_zgate"] = cat("chan_zgate", np.full(nsk, zg), np.full(nx, zg))
    a["chan_ca_depend"] = cat("chan_ca_depend", np.arange(n), np.full(nx, -1))
    out = CellModel(seed=0, gates=gates, gates2d=[], meta=m.meta, **a)
    ext = np.arange(len(m.chan_compt) + nsk, len(m.chan_compt) + extra)
    return out, ext


def stim_values(n):
    """Per-step drive sequences, 0 at reinit."""
    T = n * DT
    return {
        "inject": (T, [0.0, 0.4e-9, 0.4e-9, 0.1e-9, 0.8e-9, 0.0, 0.6e-9]),
        "conc": (T, [0.0, 0.02, 0.08, 0.0, 0.0, 0.05, 0.12, 0.03]),
        "ica": (T, [0.0, 0.0, 2e-12, 4e-12, 0.0, 0.0, 3e-12, 0.0]),
    }


def make():
    import moose
    m, ext = msg_cell()
    comp, pools, chans, handlers, gens = build_moose(m, DT)
    for t in range(8):
        moose.setClock(t, DT)
    moose.setClock(8, DT * STRIDE)
    sent = {}
    rec = {}
    for name, (T, vec) in stim_values(NSTEPS).items():
        st = moose.StimulusTable("/cell/stim_" + name)
        st.vector = vec
        st.startTime, st.stopTime, st.stepSize = 0.0, T, 0.0
        if name == "inject":
            moose.connect(st, "output", comp[0], "injectMsg")
        elif name == "conc":
            for k in ext:
                moose.connect(st, "output", chans[k], "concen")
        else:
            moose.connect(st, "output", pools[0], "current")
        t = moose.Table("/cell/sent_" + name)
        moose.connect(st, "output", t, "input")
        sent[name] = t
    rec_c = [0, 7, 19, m.n_compt - 1]
    rec_p = [0, 7, 19]
    vt, ct = [], []
    for i in rec_c:
        t = moose.Table("/cell/vm%d" % i)
        moose.connect(t, "requestOut", comp[i], "getVm")
        vt.append(t)
    for p in rec_p:
        t = moose.Table("/cell/ca%d" % p)
        moose.connect(t, "requestOut", pools[p], "getCa")
        ct.append(t)
    h = moose.HSolve("/cell/hsolve")
    h.dt = DT
    h.target = comp[m.seed].path
    moose.reinit()
    moose.start(NSTEPS * DT)
    out = dict(dt=DT, nsteps=NSTEPS, stride=STRIDE, rec=np.array(rec_c), rec_pool=np.array(rec_p), ext=ext,
               vm=np.array([t.vector for t in vt]), ca=np.array([t.vector for t in ct]),
               final_vm=np.array([c.Vm for c in comp]),
               grid=np.array([h.vMin, h.vMax, h.vDiv, h.caMin, h.caMax, h.caDiv]))
    for name, t in sent.items():
        out["sent_" + name] = np.array(t.vector)
    out.update(save_model(m))
    np.savez_compressed(os.path.join(HERE, "active_msgs.npz"), **out)
    print("wrote", os.path.join(HERE, "active_msgs.npz"), {k: out["sent_" + k].shape for k in sent})


if __name__ == "__main__":
    make()
