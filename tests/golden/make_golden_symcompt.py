#!/usr/bin/env python3
"""A branched SymCompartment cell under the reference HSolve.

HSolve takes over SymCompartments (hsolve/HSolve.cpp:505-513) and finds
their tree through distalOut, proximalOut and cylinderOut
(hsolve/HSolveUtils.cpp:36-53).  Built here in the reference build's
pymoose, with every kind of SymCompartment link that makes a tree:
  * distal -> proximal (dendrites, one branch point with two children and
    no sibling messages -- ReadCell would add them, and the reference's
    tree walk cannot take those),
  * sphere -> proximalOnly (a second primary dendrite on the soma),
  * cylinder -> proximalOnly (two spines on one dendrite),
with the GENESIS golden library's HH Na and K in every compartment, a
SpikeGen on the soma and a 0.4 nA soma inject; seeded passive values.

Just before moose.reinit() the MOOSE-side binding (hsb_fill_cell_desc,
moose-core_gb300/cpp/moose_hsolve_bridge.cpp, linked into the reference
build) describes the set-up solver; that description is saved as the
model.  Then 4,000 steps of 25 us: Vm of four compartments every 20th
step (reference Tables), spike times, the final Vm of every compartment,
and each recorded compartment's index in the description.

Output: tests/golden/symcompt_branched.npz.  Prerequisite: the reference
build (python oracle/build_ref.py).
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
sys.path.insert(0, os.path.join(REPO, "moose-core_gb300"))

from loader import model_from_desc  # noqa: E402
from make_golden_active import save_model  # noqa: E402
from make_golden_genesis import build_reference_library, library  # noqa: E402
from moose_gb300.abi import HsCellDesc  # noqa: E402

DT, NSTEPS, STRIDE, INJECT = 25e-6, 4000, 20, 0.4e-9

# name, parent, link kind (distal / sphere / cylinder), length um, diameter um
TREE = [("soma", None, None, 20.0, 20.0),
        ("d1", "soma", "distal", 12.0, 2.5),
        ("d2", "d1", "distal", 10.0, 2.0),
        ("d3", "d2", "distal", 10.0, 1.6),
        ("b1", "d1", "distal", 9.0, 1.4),     # d1's second child: a branch point
        ("b2", "b1", "distal", 9.0, 1.2),
        ("p1", "soma", "sphere", 15.0, 2.2),  # second primary dendrite
        ("p2", "p1", "distal", 15.0, 1.8),
        ("sp1", "d2", "cylinder", 1.0, 0.5),  # spines on d2
        ("sp2", "d2", "cylinder", 1.2, 0.5)]


def build(moose, rng):
    build_reference_library(library())
    cell = moose.Neutral("/symcell")
    comps = {}
    for name, par, link, L, d in TREE:
        c = moose.SymCompartment("%s/%s" % (cell.path, name))
        L, d = L * 1e-6, d * 1e-6
        area = np.pi * d * L
        c.length, c.diameter = L, d
        c.Ra = float(rng.uniform(0.8, 1.5)) * L * 4.0 / (np.pi * d * d)
        c.Rm = float(rng.uniform(1.0, 2.0)) / area
        c.Cm = 0.01 * area
        c.Em = float(rng.uniform(-0.070, -0.060))
        c.initVm = -0.065
        c.Vm = -0.065
        comps[name] = c
        if par is not None:
            src = {"distal": "distal", "sphere": "sphere", "cylinder": "cylinder"}[link]
            dst = "proximal" if link == "distal" else "proximalOnly"
            moose.connect(comps[par], src, c, dst, "Single")
        for ch, dens in (("Na", 1200.0), ("K", 360.0)):
            h = moose.copy("/library/" + ch, c, ch)
            h = moose.element(h)
            h.Gbar = dens * float(rng.uniform(0.8, 1.2)) * area
            moose.connect(c, "channel", h, "channel")
    sg = moose.SpikeGen(cell.path + "/soma/spike")
    sg.threshold, sg.refractT, sg.edgeTriggered = 0.0, 2e-3, 1
    moose.connect(comps["soma"], "VmOut", sg, "Vm")
    comps["soma"].inject = INJECT
    return cell, comps, sg


def main():
    import moose
    rng = np.random.default_rng(31)
    cell, comps, sg = build(moose, rng)
    for t in range(8):
        moose.setClock(t, DT)
    moose.setClock(8, DT * STRIDE)
    rec_names = ["soma", "d3", "b2", "sp1"]
    tabs = []
    for n in rec_names:
        t = moose.Table("%s/vm_%s" % (cell.path, n))
        moose.connect(t, "requestOut", comps[n], "getVm")
        tabs.append(t)
    spk = moose.Table(cell.path + "/spikes")
    moose.connect(sg, "spikeOut", spk, "input")
    h = moose.HSolve(cell.path + "/hsolve")
    h.dt = DT
    h.target = comps["soma"].path
    # the description of the set-up solver, by the MOOSE-side binding
    L = C.CDLL(moose._moose.__file__)
    L.hsb_fill_cell_desc.restype = C.POINTER(HsCellDesc)
    L.hsb_fill_cell_desc.argtypes = [C.c_char_p, C.POINTER(C.c_uint32)]
    L.hsb_free_cell_desc.argtypes = [C.POINTER(HsCellDesc)]
    L.hsb_object_path.argtypes = [C.POINTER(HsCellDesc), C.c_int, C.c_uint32, C.c_char_p, C.c_uint32]
    L.hsb_last_error.restype = C.c_char_p
    seed = C.c_uint32()
    d = L.hsb_fill_cell_desc(h.path.encode(), C.byref(seed))
    assert d, L.hsb_last_error()
    m = model_from_desc(d.contents, seed.value)
    buf = C.create_string_buffer(512)
    paths = []
    for i in range(d.contents.n_compt):
        assert L.hsb_object_path(d, 0, i, buf, 512) >= 0
        paths.append(buf.value.decode())
    L.hsb_free_cell_desc(d)
    index = {p.split("/")[-1].split("[")[0]: i for i, p in enumerate(paths)}
    assert sorted(index) == sorted(n for n, *_ in TREE), paths
    moose.reinit()
    moose.start(NSTEPS * DT)
    vm = np.array([t.vector for t in tabs])
    final = np.array([comps[n].Vm for n, *_ in TREE])
    spikes = np.array(spk.vector)
    print("model: %d compartments, %d channels; %d spikes; parent %s"
          % (m.n_compt, len(m.chan_compt), len(spikes), list(m.parent)))
    np.savez_compressed(os.path.join(HERE, "symcompt_branched.npz"),
                        dt=DT, nsteps=NSTEPS, stride=STRIDE, vm=vm, spikes=spikes,
                        rec=np.array([index[n] for n in rec_names]),
                        final_names=np.array([n for n, *_ in TREE]),
                        final_index=np.array([index[n] for n, *_ in TREE]), final_vm=final,
                        **save_model(m))
    print("wrote", os.path.join(HERE, "symcompt_branched.npz"))


if __name__ == "__main__":
    main()
