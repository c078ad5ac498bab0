#!/usr/bin/env python3
"""Active golden traces from the reference ``moose`` module (with HSolve).

A ``CellModel`` (``moose-core_gb300/moose_gb300/abi.py``) is translated into
reference MOOSE objects: Compartments joined by axial/raxial messages in
increasing child index; HHChannels copied from /library prototypes (so their
gates are shared, as HSolve's `gates(getOriginals)` expects); CaConcs fed by
IkOut; HHChannel2D with VOLT_C1_INDEX reading Vm and the pool's concOut;
SynChans with a SimpleSynHandler whose events are queued after reinit;
SpikeGens; Tables on tick 8.  An HSolve with target = the seed compartment
takes the cell over.  The model itself is saved beside the traces
(``model_*`` keys) so that tests rebuild it bit for bit on any machine.

Run by ``make_golden.py`` (which documents the prerequisites).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
sys.path.insert(0, os.path.join(REPO, "moose-core_gb300"))

from moose_gb300 import models  # noqa: E402
from moose_gb300.abi import HS_DEP, CellModel, _ARRAYS  # noqa: E402

DEP_NAME = {v: k for k, v in HS_DEP.items()}


def save_model(m, prefix="model_"):
    out = {prefix + "seed": np.array(m.seed)}
    for k in _ARRAYS:
        out[prefix + k] = getattr(m, k)
    out[prefix + "ngates"] = np.array(len(m.gates))
    for i, (mn, mx, A, B) in enumerate(m.gates):
        out[prefix + "gate%d" % i] = np.stack([np.asarray(A), np.asarray(B)])
        out[prefix + "gate%d_range" % i] = np.array([mn, mx])
    for k, v in m.meta.items():
        out["meta_" + k] = np.asarray(v)
    out[prefix + "ngates2d"] = np.array(len(m.gates2d))
    for i, (xmn, xmx, ymn, ymx, A, B) in enumerate(m.gates2d):
        out[prefix + "gate2d%d" % i] = np.stack([A, B])
        out[prefix + "gate2d%d_range" % i] = np.array([xmn, xmx, ymn, ymx])
    return out


def synapse(sh, j):
    """Synapse j of a SimpleSynHandler (by path: indexing the handler's
    `synapse` field does not convert in every pymoose build)."""
    import moose
    return moose.element("%s/synapse[%d]" % (sh.path, j))


def build_moose(m, dt, cell="/cell", library="/library"):
    """`library`: where the channel prototypes go (copied channels share
    their prototype's gates, so cells built side by side need their own)."""
    import moose
    for p in (cell, library):
        if moose.exists(p):
            moose.delete(p)
    moose.Neutral(library)
    root = moose.Neutral(cell)
    n = m.n_compt
    comp = []
    for i in range(n):
        c = moose.Compartment("%s/c%d" % (cell, i))
        c.Ra, c.Rm, c.Cm, c.Em = m.Ra[i], m.Rm[i], m.Cm[i], m.Em[i]
        c.initVm, c.Vm, c.inject = m.initVm[i], m.Vm[i], m.inject[i]
        comp.append(c)
    for i in range(n):
        if m.parent[i] >= 0:
            moose.connect(comp[m.parent[i]], "axial", comp[i], "raxial")
    for k in range(len(m.leak_compt)):
        lk = moose.Leakage("%s/c%d/leak%d" % (cell, m.leak_compt[k], k))
        lk.Ek, lk.Gk = m.leak_Ek[k], m.leak_Gk[k]
        moose.connect(lk, "channel", comp[m.leak_compt[k]], "channel")
    # one prototype channel per distinct gate signature
    protos = {}

    def proto(k):
        sig = (m.chan_Xpower[k], m.chan_Ypower[k], m.chan_Zpower[k], m.chan_xgate[k],
               m.chan_ygate[k], m.chan_zgate[k], m.chan_use_conc[k])
        if sig in protos:
            return protos[sig]
        p = moose.HHChannel("%s/proto%d" % (library, len(protos)))
        p.Xpower, p.Ypower, p.Zpower = m.chan_Xpower[k], m.chan_Ypower[k], m.chan_Zpower[k]
        p.useConcentration = int(m.chan_use_conc[k])
        for name, pw, g in (("gateX", m.chan_Xpower[k], m.chan_xgate[k]),
                            ("gateY", m.chan_Ypower[k], m.chan_ygate[k]),
                            ("gateZ", m.chan_Zpower[k], m.chan_zgate[k])):
            if pw > 0:
                mn, mx, A, B = m.gates[g]
                gate = moose.element(p.path + "/" + name)
                gate.min, gate.max, gate.divs = mn, mx, len(A) - 1
                gate.tableA = np.asarray(A, float)
                gate.tableB = np.asarray(B, float)
        protos[sig] = p
        return p

    pools = []
    for p in range(len(m.pool_compt)):
        ca = moose.CaConc("%s/c%d/ca%d" % (cell, m.pool_compt[p], p))
        ca.CaBasal = m.pool_CaBasal[p]
        ca.Ca = m.pool_Ca[p]
        ca.tau = m.pool_tau[p]
        ca.B = m.pool_B[p]
        ca.ceiling = m.pool_ceiling[p]
        ca.floor = m.pool_floor[p]
        if "pool_diameter" in m.meta:
            # zombification recomputes B from these (CaConcBase::updateDimensions)
            ca.thick = m.meta["pool_thick"][p]
            ca.length = m.meta["pool_length"][p]
            ca.diameter = m.meta["pool_diameter"][p]
        pools.append(ca)
    chans = []
    for k in range(len(m.chan_compt)):
        ch = moose.copy(proto(k), comp[m.chan_compt[k]], "chan%d" % k)
        ch = moose.element(ch)
        ch.Gbar, ch.Ek = m.chan_Gbar[k], m.chan_Ek[k]
        ch.instant = int(m.chan_instant[k])
        ch.modulation = m.chan_modulation[k]
        if m.chan_Xpower[k] > 0:
            ch.X = m.chan_X[k]
        if m.chan_Ypower[k] > 0:
            ch.Y = m.chan_Y[k]
        if m.chan_Zpower[k] > 0:
            ch.Z = m.chan_Z[k]
        moose.connect(ch, "channel", comp[m.chan_compt[k]], "channel")
        if m.chan_ca_target[k] >= 0:
            moose.connect(ch, "IkOut", pools[m.chan_ca_target[k]], "current")
        if m.chan_ca_depend[k] >= 0:
            moose.connect(pools[m.chan_ca_depend[k]], "concOut", ch, "concen")
        chans.append(ch)
    # HHChannel2D after the HHChannels; SynChans after them (tick-4 order)
    protos2d = {}
    for k in range(len(m.c2d_compt)):
        g = int(m.c2d_xgate[k])
        if g not in protos2d:
            p = moose.HHChannel2D("%s/proto2d%d" % (library, g))
            p.Xindex = DEP_NAME[int(m.c2d_xindex[k])]
            p.Xpower = m.c2d_Xpower[k]
            xmn, xmx, ymn, ymx, A, B = m.gates2d[g]
            gate = moose.element(p.path + "/gateX")
            gate.tableA = np.asarray(A, float).tolist()
            gate.tableB = np.asarray(B, float).tolist()
            gate.xmin, gate.xmax = xmn, xmx
            gate.ymin, gate.ymax = ymn, ymx
            protos2d[g] = p
        ch = moose.element(moose.copy(protos2d[g], comp[m.c2d_compt[k]], "kca%d" % k))
        ch.Gbar, ch.Ek = m.c2d_Gbar[k], m.c2d_Ek[k]
        if m.c2d_instant[k]:          # HHChannel2D has no `instant` field
            raise ValueError("instant HHChannel2D gates are not expressible in MOOSE")
        ch.modulation = m.c2d_modulation[k]
        # no X field: reinit sets X = A/B at the default inputs (Vm = 0, conc = 0)
        if m.c2d_X[k] != 0.0:
            raise ValueError("HHChannel2D initial X must be 0 for the reference")
        moose.connect(ch, "channel", comp[m.c2d_compt[k]], "channel")
        moose.connect(comp[m.c2d_compt[k]], "VmOut", ch, "Vm")
        if m.c2d_conc1_pool[k] >= 0:
            moose.connect(pools[m.c2d_conc1_pool[k]], "concOut", ch, "concen")
        if m.c2d_conc2_pool[k] >= 0:
            moose.connect(pools[m.c2d_conc2_pool[k]], "concOut", ch, "concen2")
    handlers = []
    for k in range(len(m.syn_compt)):
        sc = moose.SynChan("%s/c%d/syn%d" % (cell, m.syn_compt[k], k))
        sc.Gbar, sc.Ek = m.syn_Gbar[k], m.syn_Ek[k]
        sc.tau1, sc.tau2 = m.syn_tau1[k], m.syn_tau2[k]
        sc.modulation = m.syn_modulation[k]
        sh = moose.SimpleSynHandler(sc.path + "/sh")
        sh.numSynapses = 1
        synapse(sh, 0).delay = 0.0
        w = np.unique(m.ev_weight[m.ev_syn == k])
        if len(w) > 1:
            raise ValueError("one synapse per SynChan: its events share one weight")
        synapse(sh, 0).weight = float(w[0]) if len(w) else 1.0
        moose.connect(sh, "activationOut", sc, "activation")
        moose.connect(sc, "channel", comp[m.syn_compt[k]], "channel")
        handlers.append(sh)
    gens = []
    for k in range(len(m.sg_compt)):
        sg = moose.SpikeGen("%s/sg%d" % (cell, k))
        sg.threshold, sg.refractT = m.sg_threshold[k], m.sg_refractT[k]
        sg.edgeTriggered = int(m.sg_edge[k])
        moose.connect(comp[m.sg_compt[k]], "VmOut", sg, "Vm")
        gens.append(sg)
    return comp, pools, chans, handlers, gens


def run_moose(m, dt, nsteps, rec_compts, rec_pools=(), stride=1, ca_advance=1,
              dt_setup=None):
    """Step `m` for nsteps under the reference HSolve; return traces and spikes."""
    import moose
    comp, pools, chans, handlers, gens = build_moose(m, dt)
    for t in range(8):
        moose.setClock(t, dt)
    moose.setClock(8, dt * stride)
    tabs = []
    for i in rec_compts:
        t = moose.Table("/cell/vm%d" % i)
        moose.connect(t, "requestOut", comp[i], "getVm")
        tabs.append(t)
    ctabs = []
    for p in rec_pools:
        t = moose.Table("/cell/ca%d" % p)
        moose.connect(t, "requestOut", pools[p], "getCa")
        ctabs.append(t)
    spk = []
    for k, g in enumerate(gens):
        t = moose.Table("/cell/spk%d" % k)
        moose.connect(g, "spikeOut", t, "input")   # Table::input stores the time sent
        spk.append(t)
    h = moose.HSolve("/cell/hsolve")
    h.dt = dt if dt_setup is None else dt_setup
    h.caAdvance = ca_advance
    h.target = comp[m.seed].path
    moose.reinit()
    # events are queued after reinit (SimpleSynHandler::vReinit clears them)
    for e in range(len(m.ev_syn)):
        synapse(handlers[m.ev_syn[e]], 0).addSpike(float(m.ev_time[e]))
    cur = 0
    sched = list(zip(m.stim_step.tolist(), m.stim_compt.tolist(), m.stim_value.tolist()))
    for step, c, v in sched + [(nsteps, None, None)]:
        step = min(step, nsteps)
        if step > cur:
            moose.start((step - cur) * dt)
            cur = step
        if c is not None and step < nsteps:
            comp[c].inject = v
    vm = np.array([t.vector for t in tabs])
    ca = np.array([t.vector for t in ctabs]) if ctabs else np.zeros((0, 0))
    spikes = [np.array(t.vector) for t in spk]
    final_vm = np.array([c.Vm for c in comp])
    return vm, ca, spikes, final_vm, h


def make_active():
    out_dir = HERE
    dt = 25e-6
    # 1. the single-cell HH cable workload, full length (0.5 s)
    m = models.config1_cell()
    rec = [0, 50, 100, 150, 200]
    vm, ca, spikes, final_vm, h = run_moose(m, dt, 20000, rec, stride=10)
    np.savez_compressed(os.path.join(out_dir, "active_hh_cable.npz"),
                        dt=dt, nsteps=20000, stride=10, rec=np.array(rec), vm=vm,
                        spikes=spikes[0], final_vm=final_vm,
                        grid=np.array([h.vMin, h.vMax, h.vDiv, h.caMin, h.caMax, h.caDiv]),
                        **save_model(m))
    print("hh_cable: samples", vm.shape, "spikes", len(spikes[0]))
    # 2. branched cell with Ca(HVA), K(Ca) 2-D gate, CaConc, SynChans, SpikeGen
    rng = np.random.default_rng(7)
    parent, d, L = models.branched_morphology(rng, 60, 0.5, 4)
    kA, kB = models.kca_2d_tables(vdivs=150, cadivs=100)
    m = models.active_cell(parent, d, L, inject=0.4e-9, n_syn=12, syn_rate=40.0, t_end=0.2,
                           rng=rng, gca=20.0, kca_tables=(kA, kB), inject_step=400)
    m.seed = 0
    rec = list(range(0, 60, 6))
    vm, ca, spikes, final_vm, h = run_moose(m, dt, 8000, rec, rec_pools=rec, stride=4)
    np.savez_compressed(os.path.join(out_dir, "active_branched_kca.npz"),
                        dt=dt, nsteps=8000, stride=4, rec=np.array(rec), vm=vm, ca=ca,
                        spikes=spikes[0], final_vm=final_vm, ca_advance=1,
                        **save_model(m))
    print("branched_kca: samples", vm.shape, "spikes", len(spikes[0]))
    # 3. same cell, caAdvance = 0, seeded from a dendrite, setup dt != clock dt
    m.seed = 17
    vm, ca, spikes, final_vm, h = run_moose(m, dt, 2000, rec, rec_pools=rec, stride=4,
                                            ca_advance=0, dt_setup=50e-6)
    np.savez_compressed(os.path.join(out_dir, "active_branched_caadv0.npz"),
                        dt=dt, dt_setup=50e-6, nsteps=2000, stride=4, rec=np.array(rec),
                        vm=vm, ca=ca, spikes=spikes[0], final_vm=final_vm, ca_advance=0,
                        **save_model(m))
    print("branched_caadv0: samples", vm.shape, "spikes", len(spikes[0]))


if __name__ == "__main__":
    make_active()
