#!/usr/bin/env python3
"""GENESIS .p cell files and what the REFERENCE builds from them.

1. A channel library (the reference's ``/library``): HH Na (m^3 h) and K
   (n^4), Ca(HVA) (m^2 h) whose ``addmsg1`` sends IkOut to the sibling
   ``Ca_conc``, an SK-type channel on concentration and a K(Ca)
   HHChannel2D on (Vm, Ca), both fed by ``Ca_conc`` through ``addmsg1``,
   a CaConc, a SpikeGen and a glu SynChan with its one-synapse handler (as
   ``rdesigneurProtos.make_glu``).  The same library is written as
   ``moose_gb300.genesis`` prototypes by ``library()`` below, which the
   tests import; its gate tables are saved with the results (``lib_*``)
   so that the tests step the very tables the reference stepped.
2. Seeded synthetic .p files under ``tests/golden/genesis/`` (trees grown
   here): relative and absolute, cartesian and polar coordinates, a
   spherical soma (length 0), ``*double_endpoint`` lines, ``*set_global`` /
   ``*set_compt_param`` changes part way, EREST_ACT / ELEAK flags, the ``.``
   parent, RA/RM/CM and Ra/Rm/Cm overrides, absolute (negative) densities,
   ``//`` and ``/* */`` comments, blank lines and tabs; an unbranched
   ``*symmetric`` cable (SymCompartments, each compartment's class saved);
   a cell with glu SynChans (density and absolute) and events queued on
   them after reinit (saved as ``ev_*``);
   and a cell of compartment prototypes (``*compt``: two prototype
   compartments in ``/library`` with copied channels, a CaConc, their
   messages and an inject; a ``*compt`` whose path is not the prototype's
   Id path, which the reference ignores).
3. Each file loaded by the reference ``moose.loadModel`` (``ReadCell``):
   every compartment (creation order: name, parent, Ra, Rm, Cm, Em, initVm,
   diameter, length, coordinates), every channel (compartment, name, Gbar,
   Ek), every SynChan (compartment, Gbar, Ek, tau1, tau2), CaConc B after
   zombification, SpikeGen threshold; then a soma inject
   of 0.3 nA and 4,000 steps of 25 us under an HSolve with target = the
   first compartment: Vm and Ca traces (every 20th step), spikes, final Vm.

Output: ``tests/golden/genesis_golden.npz``.  Prerequisite: the reference
build (``python oracle/build_ref.py``).
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "moose-core_gb300"))
P_DIR = os.path.join(HERE, "genesis")
DT, NSTEPS, STRIDE, INJECT = 25e-6, 4000, 20, 0.3e-9

from moose_gb300 import genesis, models  # noqa: E402


def _sk_gate(cmax=0.1, cdivs=400, kd=0.02, tau=5e-3):
    c = np.linspace(0.0, cmax, cdivs + 1)
    zinf = c ** 4 / (c ** 4 + kd ** 4)
    return (0.0, cmax, zinf / tau, np.full_like(c, 1.0 / tau))


def _tables(z=None):
    """Gate tables of the library: computed here (numpy exp, whose last bit
    can differ between machines) or read back from the golden file, so that
    every machine steps the tables the reference stepped."""
    names = ("mA", "mB", "hA", "hB", "nA", "nB", "cxA", "cxB", "cyA", "cyB", "kA", "kB", "skA", "skB")
    if z is not None:
        return {k: z["lib_" + k] for k in names}
    (mA, mB), (hA, hB) = models.hh_na_tables()
    nA, nB = models.hh_k_tables()
    (cxA, cxB), (cyA, cyB) = models.ca_hva_tables()
    kA, kB = models.kca_2d_tables(vdivs=300, cadivs=300)
    _, _, skA, skB = _sk_gate()
    v = locals()
    return {k: v[k] for k in names}


def library(z=None):
    """The channel library as moose_gb300.genesis prototypes (tables from
    the golden file `z` when given), with the compartment prototypes."""
    lib = _channel_library(z)
    lib.update(compartment_protos(lib))
    return lib


def _channel_library(z=None):
    V = (models.VMIN, models.VMAX)
    t = _tables(z)
    mA, mB, hA, hB, nA, nB = t["mA"], t["mB"], t["hA"], t["hB"], t["nA"], t["nB"]
    cxA, cxB, cyA, cyB, kA, kB = t["cxA"], t["cxB"], t["cyA"], t["cyB"], t["kA"], t["kB"]
    sk = _sk_gate()[:2] + (t["skA"], t["skB"])
    return {
        "Na": genesis.HHChannelProto(Ek=0.05, Xpower=3, Ypower=1, xgate=V + (mA, mB), ygate=V + (hA, hB)),
        "K": genesis.HHChannelProto(Ek=-0.077, Xpower=4, xgate=V + (nA, nB)),
        "CaHVA": genesis.HHChannelProto(Ek=0.08, Xpower=2, Ypower=1, xgate=V + (cxA, cxB), ygate=V + (cyA, cyB),
                                        addmsg=[". IkOut ../Ca_conc current"]),
        "SK": genesis.HHChannelProto(Ek=-0.077, Zpower=1, zgate=sk, useConcentration=1,
                                     addmsg=["../Ca_conc concOut . concen"]),
        "KCa": genesis.HHChannel2DProto(Ek=-0.077, Xpower=1,
                                        table=(models.VMIN, models.VMAX, models.CAMIN, models.CAMAX, kA, kB),
                                        addmsg=["../Ca_conc concOut . concen"]),
        "Ca_conc": genesis.CaConcProto(tau=0.02, CaBasal=5e-5, thick=0.1e-6, diameter=2e-6, length=10e-6),
        "spike": genesis.SpikeGenProto(refractT=2e-3, edgeTriggered=1),
        "glu": genesis.SynChanProto(Ek=0.0, tau1=2e-3, tau2=9e-3, weight=1.0),
    }


def compartment_protos(lib):
    """Compartment prototypes for ``*compt`` (built in the reference's
    /library by build_reference_library): children copied from the
    library with absolute conductances, their messages and an inject."""
    return {
        "protoSoma": genesis.CompartmentProto(
            children=[("K", lib["K"], {"Gbar": 3.1e-7}), ("Na", lib["Na"], {"Gbar": 1.25e-6}),
                      ("CaHVA", lib["CaHVA"], {"Gbar": 4.5e-9}), ("Ca_conc", lib["Ca_conc"], {}),
                      ("SK", lib["SK"], {"Gbar": 2.2e-9})],
            msgs=[("CaHVA", "IkOut", "Ca_conc", "current"), ("Ca_conc", "concOut", "SK", "concen")]),
        "protoDend": genesis.CompartmentProto(
            children=[("CaHVA", lib["CaHVA"], {"Gbar": 1.3e-9}), ("Ca_conc", lib["Ca_conc"], {}),
                      ("K", lib["K"], {"Gbar": 6.5e-8})],
            msgs=[("CaHVA", "IkOut", "Ca_conc", "current")], inject=4e-12),
    }


def build_reference_library(lib):
    import moose
    if moose.exists("/library"):
        moose.delete("/library")
    moose.Neutral("/library")
    for name, p in lib.items():
        path = "/library/" + name
        if isinstance(p, genesis.HHChannelProto):
            ch = moose.HHChannel(path)
            ch.Ek = p.Ek
            ch.Xpower, ch.Ypower, ch.Zpower = p.Xpower, p.Ypower, p.Zpower
            ch.useConcentration = p.useConcentration
            for gname, g in (("gateX", p.xgate), ("gateY", p.ygate), ("gateZ", p.zgate)):
                if g is not None:
                    gate = moose.element(path + "/" + gname)
                    gate.min, gate.max, gate.divs = g[0], g[1], len(g[2]) - 1
                    gate.tableA = np.asarray(g[2], float)
                    gate.tableB = np.asarray(g[3], float)
        elif isinstance(p, genesis.HHChannel2DProto):
            ch = moose.HHChannel2D(path)
            ch.Ek = p.Ek
            ch.Xindex = p.Xindex
            ch.Xpower = p.Xpower
            xmn, xmx, ymn, ymx, A, B = p.table
            gate = moose.element(path + "/gateX")
            gate.tableA = np.asarray(A, float).tolist()
            gate.tableB = np.asarray(B, float).tolist()
            gate.xmin, gate.xmax, gate.ymin, gate.ymax = xmn, xmx, ymn, ymx
        elif isinstance(p, genesis.CaConcProto):
            ch = moose.CaConc(path)
            ch.tau, ch.CaBasal, ch.Ca = p.tau, p.CaBasal, p.CaBasal
            ch.ceiling, ch.floor = p.ceiling, p.floor
            ch.thick, ch.length, ch.diameter = p.thick, p.length, p.diameter
        elif isinstance(p, genesis.SpikeGenProto):
            ch = moose.SpikeGen(path)
            ch.refractT, ch.edgeTriggered = p.refractT, p.edgeTriggered
        elif isinstance(p, genesis.SynChanProto):
            # as rdesigneurProtos.make_glu: the SynChan and a one-synapse handler
            ch = moose.SynChan(path)
            ch.Ek, ch.tau1, ch.tau2 = p.Ek, p.tau1, p.tau2
            sh = moose.SimpleSynHandler(path + "/sh")
            moose.connect(sh, "activationOut", ch, "activation")
            sh.numSynapses = 1
            moose.element(sh.path + "/synapse[0]").weight = p.weight
        elif isinstance(p, genesis.CompartmentProto):
            # children copied from the library entries, in message order
            pc = moose.SymCompartment(path) if p.symmetric else moose.Compartment(path)
            pc.inject = p.inject
            kids = {}
            for cname, cp, f in p.children:
                src = next(k for k, v in lib.items() if v is cp)
                e = moose.element(moose.copy("/library/" + src, pc, cname))
                for k, v in f.items():
                    setattr(e, k, v)
                if isinstance(cp, (genesis.HHChannelProto, genesis.HHChannel2DProto)):
                    moose.connect(pc, "channel", e, "channel")
                elif isinstance(cp, genesis.SpikeGenProto):
                    moose.connect(pc, "VmOut", e, "Vm")
                kids[cname] = e
            for s, sf, d, df in p.msgs:
                moose.connect(kids[s], sf, kids[d], df)
            continue
        for k, v in enumerate(getattr(p, "addmsg", ())):
            ms = moose.Mstring(path + "/addmsg%d" % (k + 1))
            ms.value = v


def synth_p(seed, n, header, chans, polar=False, relative=True, double_every=0, spherical_soma=False,
            midfile=None, overrides=False, after_soma=()):
    """A .p file: a seeded tree of n compartments below a soma."""
    rng = np.random.default_rng(seed)
    out = ["// synthetic GENESIS cell, seed %d" % seed, "/* header comment", "   spans lines */"]
    out += header
    out.append("*start_cell")
    soma = "soma none 0 0 0 18" if spherical_soma else "soma none 18 0 0 18"
    out.append(soma + "  " + chans(0, rng))
    out += list(after_soma)
    names, pos = ["soma"], [np.array([0.0, 0.0, 0.0]) if spherical_soma else np.array([18.0, 0.0, 0.0])]
    tips = [0, 0, 0]
    last = 0
    for i in range(1, n):
        if midfile and i == n // 2:
            out += midfile
        if rng.random() < 0.5 and last in tips:
            p = last
            tips.remove(last)
        else:
            p = tips.pop(int(rng.integers(len(tips))))
        step = rng.uniform(3.0, 12.0)
        d = rng.uniform(0.6, 2.5)
        th, ph = rng.uniform(0, 360), rng.uniform(20, 160)
        rr = np.radians
        v = step * np.array([np.sin(rr(ph)) * np.cos(rr(th)), np.sin(rr(ph)) * np.sin(rr(th)), np.cos(rr(ph))])
        pos.append(pos[p] + v)
        name = "d%d" % i
        par = "." if p == last and rng.random() < 0.6 else names[p]
        if polar:
            xyz = (v if relative else pos[-1])
            r = np.linalg.norm(xyz)
            coords = [r, np.degrees(np.arctan2(xyz[1], xyz[0])), np.degrees(np.arccos(xyz[2] / r))]
        else:
            coords = list(v if relative else pos[-1])
        fmt = lambda a: " ".join("%.5g" % x for x in a)
        line = "%s %s " % (name, par)
        if double_every and i % double_every == 0:
            start = (np.zeros(3) if relative else pos[p])
            if polar:
                # the start point at the parent's end point (absolute) or at 0 (relative)
                start = [0.0, 0.0, 0.0] if relative else [np.linalg.norm(pos[p]), np.degrees(
                    np.arctan2(pos[p][1], pos[p][0])), np.degrees(np.arccos(pos[p][2] / max(np.linalg.norm(pos[p]), 1e-9)))]
            line = "%s %s " % (name, par)
            out.append("*double_endpoint")
            out.append(line + fmt(start) + " " + fmt(coords) + " %.4g " % d + chans(i, rng))
            out.append("*double_endpoint_off")
        else:
            sep = "\t" if rng.random() < 0.15 else " "
            line = sep.join([name, par, fmt(coords), "%.4g" % d]) + "  " + chans(i, rng)
            if overrides and rng.random() < 0.1:
                line += " " + ["RA 2.5", "RM 0.5", "CM 0.02", "Ra 1.5e7", "Rm 3e9", "Cm 4e-12"][int(rng.integers(6))]
            if rng.random() < 0.1:
                line += "   // trailing comment"
            out.append(line)
        if rng.random() < 0.05:
            out.append("")
        names.append(name)
        tips.append(i)
        last = i
    return "\n".join(out) + "\n"


def chain_p(seed, n, header, chans):
    """A .p file: a soma and an unbranched dendrite of n - 1 compartments."""
    rng = np.random.default_rng(seed)
    out = ["// synthetic GENESIS cable, seed %d" % seed] + header + ["*start_cell"]
    out.append("soma none 18 0 0 18  " + chans(0, rng))
    for i in range(1, n):
        v = rng.uniform(3.0, 12.0) * np.array([1.0, rng.uniform(-0.3, 0.3), rng.uniform(-0.3, 0.3)])
        par = "." if i > 1 and rng.random() < 0.5 else ("soma" if i == 1 else "d%d" % (i - 1))
        out.append("d%d %s %.5g %.5g %.5g %.4g  %s" % (i, par, v[0], v[1], v[2], rng.uniform(0.8, 2.5), chans(i, rng)))
    return "\n".join(out) + "\n"


def _chans_hh(i, rng):
    return "Na 1200 K 360"


def _chans_full(i, rng):
    na = "Na -2e-09" if i % 7 == 5 else "Na %g" % (1200 * rng.uniform(0.8, 1.2))   # absolute or density
    s = "%s K %g CaHVA %g Ca_conc 5.2e-6 SK %g" % (na, 360, 8.0, 30.0)
    if i % 3 == 0:
        s += " KCa 40"
    if i == 0:
        s += " spike 0.0"
    return s


def _chans_proto(i, rng):
    """Line channels on top of the prototypes' children (no name twice)."""
    if i == 0:
        return "KCa 40 spike 0.0"
    s = "Na -2e-09" if i % 5 == 2 else "Na %g" % (900 * rng.uniform(0.8, 1.2))
    return s + (" KCa 30" if i % 3 == 0 else "")


def _chans_syn(i, rng):
    """HH channels and, on most compartments, a glu SynChan (density, or
    absolute on a few)."""
    s = "Na 1200 K 360"
    if i % 4 == 1:
        s += " glu -2e-10"
    elif i % 4 != 3:
        s += " glu %g" % (8.0 * rng.uniform(0.5, 1.5))
    return s + (" spike 0.0" if i == 0 else "")


def _chans_abs(i, rng):
    return "Na %g K -%g" % (1000.0, 3e-9 * rng.uniform(0.5, 1.5)) + (" spike -0.01" if i == 0 else "")


def fixtures():
    return {
        "relative_cartesian": synth_p(21, 60, ["*relative", "*cartesian", "*asymmetric", "*set_global RM 2.0",
                                               "*set_global RA 1.5", "*set_global CM 0.012",
                                               "*set_global EREST_ACT -0.068"], _chans_full, overrides=True),
        "absolute_polar": synth_p(22, 50, ["*absolute", "*polar", "*set_compt_param ELEAK -0.055"], _chans_abs,
                                  polar=True, relative=False, double_every=9,
                                  midfile=["*set_compt_param RM 3.5", "*set_global CM 0.02"]),
        "spherical_soma": synth_p(23, 40, ["*relative", "*cartesian", "*set_global EREST_ACT -0.07",
                                           "*set_global ELEAK -0.06"], _chans_hh, spherical_soma=True,
                                  double_every=11),
        # SymCompartments (distal -> proximal messages; unbranched, so no
        # sibling messages, which the reference's tree walk cannot take)
        "symmetric_cable": chain_p(24, 45, ["*relative", "*cartesian", "*symmetric", "*set_global RM 1.5",
                                            "*set_global RA 1.2"], _chans_full),
        # compartment prototypes: the soma a copy of protoSoma, the rest of
        # protoDend; the *compt half way names the prototype by a path that
        # is not its Id::path, so the reference warns and keeps protoDend
        # glu SynChans (ReadCell's canonical channels) with queued events
        "synapses": synth_p(26, 40, ["*relative", "*cartesian", "*set_global RM 1.8"], _chans_syn),
        "compt_proto": synth_p(25, 36, ["*relative", "*cartesian", "*set_global RM 2.5",
                                        "*compt /library[0]/protoSoma"], _chans_proto,
                               after_soma=["*compt /library[0]/protoDend"],
                               midfile=["*compt /library/protoSoma", "*set_global CM 0.015"]),
    }


def make():
    sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
    import moose
    lib = library()
    os.makedirs(P_DIR, exist_ok=True)
    out = {}
    for k, (name, text) in enumerate(sorted(fixtures().items())):
        path = os.path.join(P_DIR, name + ".p")
        with open(path, "w") as f:
            f.write(text)
        build_reference_library(lib)
        where = "/gcell%d" % k
        moose.loadModel(path, where)
        cs = moose.wildcardFind(where + "/#[ISA=CompartmentBase]")
        cs.sort(key=lambda c: int(re.search(r"id=(\d+)", str(c.id)).group(1)))
        names = [c.name for c in cs]
        idx = {c: i for i, c in enumerate(names)}
        out[name + "/names"] = np.array(names)
        # the parent: the raxial source (Compartment) or the proximal end (SymCompartment)
        up = [c.neighbors["proximalOut"] if c.className == "SymCompartment" else c.neighbors["raxial"] for c in cs]
        out[name + "/parent"] = np.array([idx[u[0].name] if len(u) else -1 for u in up], np.int32)
        out[name + "/classes"] = np.array([c.className for c in cs])
        for f in ("Ra", "Rm", "Cm", "Em", "initVm", "diameter", "length", "x0", "y0", "z0", "x", "y", "z"):
            out[name + "/" + f] = np.array([getattr(c, f) for c in cs], np.float64)
        chans = []
        for i, c in enumerate(cs):
            for ch in c.neighbors["channel"]:
                e = moose.element(ch)
                if e.className in ("HHChannel", "HHChannel2D"):
                    chans.append((i, e.name, e.Gbar, e.Ek))
        out[name + "/chan_compt"] = np.array([x[0] for x in chans], np.int32)
        out[name + "/chan_name"] = np.array([x[1] for x in chans])
        out[name + "/chan_Gbar"] = np.array([x[2] for x in chans])
        out[name + "/chan_Ek"] = np.array([x[3] for x in chans])
        sgs = moose.wildcardFind(where + "/##[ISA=SpikeGen]")
        out[name + "/sg_threshold"] = np.array([s.threshold for s in sgs])
        syns = moose.wildcardFind(where + "/##[ISA=SynChan]")
        syns.sort(key=lambda c: int(re.search(r"id=(\d+)", str(c.id)).group(1)))
        out[name + "/syn_compt"] = np.array([idx[moose.element(s.neighbors["channel"][0]).name] for s in syns],
                                            np.int32)
        for f in ("Gbar", "Ek", "tau1", "tau2"):
            out[name + "/syn_" + f] = np.array([getattr(s, f) for s in syns], np.float64)
        for t in range(8):
            moose.setClock(t, DT)
        moose.setClock(8, DT * STRIDE)
        soma = cs[0]
        soma.inject = INJECT
        rec = [0, len(cs) // 2, len(cs) - 1]
        vt = []
        for i in rec:
            t = moose.Table("%s/vm%d" % (where, i))
            moose.connect(t, "requestOut", cs[i], "getVm")
            vt.append(t)
        pools = moose.wildcardFind(where + "/##[ISA=CaConcBase]")
        pools.sort(key=lambda c: int(re.search(r"id=(\d+)", str(c.id)).group(1)))
        ct = []
        for i in range(min(3, len(pools))):
            t = moose.Table("%s/ca%d" % (where, i))
            moose.connect(t, "requestOut", pools[i], "getCa")
            ct.append(t)
        st = []
        for i, s in enumerate(sgs):
            t = moose.Table("%s/spk%d" % (where, i))
            moose.connect(s, "spikeOut", t, "input")
            st.append(t)
        h = moose.HSolve(where + "/hsolve")
        h.dt = DT
        h.target = soma.path
        moose.reinit()
        # synaptic events, queued after reinit (SimpleSynHandler::vReinit
        # drops earlier ones): SynChan k gets six, 11 ms apart
        ev = [(k, 0.004 + 0.0031 * k + 0.011 * j) for k in range(len(syns)) for j in range(6)]
        for k, t in ev:
            moose.element(syns[k].path + "/sh/synapse[0]").addSpike(t)
        if syns:
            out[name + "/ev_syn"] = np.array([k for k, _ in ev], np.uint32)
            out[name + "/ev_time"] = np.array([t for _, t in ev])
            out[name + "/ev_weight"] = np.array([moose.element(syns[k].path + "/sh/synapse[0]").weight
                                                 for k, _ in ev])
        moose.start(NSTEPS * DT)
        out[name + "/pool_B"] = np.array([p.B for p in pools])
        out[name + "/vm"] = np.array([t.vector for t in vt])
        out[name + "/ca"] = np.array([t.vector for t in ct]) if ct else np.zeros((0, 0))
        out[name + "/spikes"] = np.array(st[0].vector) if st else np.zeros(0)
        out[name + "/final_vm"] = np.array([c.Vm for c in cs])
        out[name + "/rec"] = np.array(rec)
        moose.delete(where)
    out.update({"lib_" + k: v for k, v in _tables().items()})
    np.savez_compressed(os.path.join(HERE, "genesis_golden.npz"), dt=DT, nsteps=NSTEPS, stride=STRIDE,
                        inject=INJECT, **out)
    print("wrote", os.path.join(HERE, "genesis_golden.npz"))


if __name__ == "__main__":
    make()
