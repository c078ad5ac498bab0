#!/usr/bin/env python3
"""rdesigneur models built by the REFERENCE's own rdesigneur, for the
rdesigneur loader (moose_gb300.rdes).

Each case calls the reference's ``rdesigneur.rdesigneur(...).buildModel()``
(python/rdesigneur/rdesigneur.py) in the reference build's pymoose.  The
package imports plotting and 3-D viewer modules that this image does not
have; empty stand-in modules are put in ``sys.modules`` for those before
the import (moose itself is imported first, without them), and nothing
here plots.  Right after buildModel, whose last steps set up the HSolve,
the MOOSE-side binding (``hsb_fill_cell_desc``) describes the solver; then
the model runs for ``t_end`` and the soma plot Table is read.

Cases:
* ``ball_and_stick``: the arguments of the reference's
  tests/rdesigneur/test_41_ballAndStick.py (read from that file);
* ``soma_pulse``: tests/rdesigneur/test_20_currentPulse.py's arguments
  (the default passive HH soma, a current pulse);
* ``branched_distrib``: a branchedCell with a passive distribution and
  channel distributions that use p, g, L, dia, maxP, exp, H, ?: and ^,
  HH Na/K, a Ca channel feeding a CaConc (IkOut) and a K_AHP reading it
  (concen), a current pulse;
* ``glu_distrib``: a branchedCell with HH Na/K and ``make_glu()`` SynChans
  distributed over the dendrites (Gbar growing with p, Ek set), a step
  current.

Saved per case (``rdes_model_<case>.npz``): the rdesigneur arguments
(JSON), the /library prototypes the model used (fields and gate tables),
the described model (``model_*``), each compartment's, channel's and
pool's path in the description, the plot Table's samples and its stride.
Prerequisite: the reference build (``python oracle/build_ref.py``).
"""
import ast
import ctypes as C
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
sys.path.insert(0, os.path.join(REPO, "moose-core_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from build_ref import source_dir  # noqa: E402
from loader import model_from_desc  # noqa: E402
from make_golden_active import save_model  # noqa: E402
from moose_gb300.abi import HsCellDesc  # noqa: E402

REF_TESTS = os.path.join(source_dir(), "tests", "rdesigneur")


def test_call(name, func):
    """The literal keyword arguments of the rdesigneur(...) call in a
    reference test function."""
    tree = ast.parse(open(os.path.join(REF_TESTS, name)).read())
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == func)
    for node in ast.walk(fn):
        if isinstance(node, ast.Call) and getattr(node.func, "attr", None) == "rdesigneur":
            return {k.arg: ast.literal_eval(k.value) for k in node.keywords}
    raise ValueError("no rdesigneur call in %s.%s" % (name, func))


CASES = {
    "ball_and_stick": lambda: dict(t_end=0.06, **{k: v for k, v in test_call(
        "test_41_ballAndStick.py", "test_ball_and_stick").items() if k != "moogList"}),
    "soma_pulse": lambda: dict(t_end=0.3, **test_call("test_20_currentPulse.py", "test_current_pulse")),
    "branched_distrib": lambda: dict(
        t_end=0.05,
        cellProto=[["branchedCell", "cell", 12e-6, 12e-6, 3e-6, 150e-6, 6, 1.5e-6, 120e-6, 5]],
        chanProto=[["make_HH_Na()", "Na"], ["make_HH_K()", "K"], ["make_Ca_conc()", "Ca_conc"],
                   ["make_Ca()", "Ca"], ["make_K_AHP()", "K_AHP"]],
        passiveDistrib=[["#", "RM", "1.0 + 2e3 * p", "CM", "0.012"], ["dend#", "RA", "1.2"],
                        ["branch#", "Em", "-0.066 + 20 * g", "initVm", "-0.067"]],
        chanDistrib=[["Na", "soma", "Gbar", "1000"],
                     ["Na", "dend#,branch#", "Gbar", "400 * exp(-p/200e-6) + 20"],
                     ["K", "#", "Gbar", "dia > 2e-6 ? 300 : 150", "Ek", "-0.08"],
                     ["Ca_conc", "#", "tau", "0.02 + 1e-2 * H(g - 50e-6)", "CaBasal", "1e-4"],
                     ["Ca", "soma,dend#", "Gbar", "20 * (L < 0.5) + 5"],
                     ["K_AHP", "#", "Gbar", "8 + 2 * (p/maxP)^2"]],
        stimList=[["soma", "1", ".", "inject", "(t>0.005 && t<0.045) * 3e-10"]],
        plotList=[["soma", "1", ".", "Vm", "soma Vm"]]),
    "glu_distrib": lambda: dict(
        t_end=0.04,
        cellProto=[["branchedCell", "cell", 15e-6, 15e-6, 3e-6, 120e-6, 4, 1.5e-6, 100e-6, 4]],
        chanProto=[["make_HH_Na()", "Na"], ["make_HH_K()", "K"], ["make_glu()", "glu"]],
        chanDistrib=[["Na", "soma", "Gbar", "1200"], ["K", "#", "Gbar", "360"],
                     ["glu", "dend#,branch#", "Gbar", "5 + 2e4 * p", "Ek", "-0.005"]],
        stimList=[["soma", "1", ".", "inject", "(t>0.004) * 2e-10"]],
        plotList=[["soma", "1", ".", "Vm", "soma Vm"]]),
}


def library(moose):
    """The /library prototypes: fields, gate tables and addmsg strings."""
    out = {}
    for e in moose.wildcardFind("/library/#"):
        cls = e.className
        d = {"class": cls}
        if cls in ("HHChannel", "ZombieHHChannel"):
            d.update(Ek=e.Ek, Gbar=e.Gbar, Xpower=e.Xpower, Ypower=e.Ypower, Zpower=e.Zpower,
                     instant=int(e.instant), useConcentration=int(e.useConcentration))
            for g in ("X", "Y", "Z"):
                if getattr(e, g + "power") > 0:
                    ge = moose.element(e.path + "/gate" + g)
                    d["gate" + g] = (ge.min, ge.max, np.array(ge.tableA), np.array(ge.tableB))
        elif cls in ("CaConc", "ZombieCaConc"):
            d.update(tau=e.tau, CaBasal=e.CaBasal, thick=e.thick, diameter=e.diameter, length=e.length,
                     ceiling=e.ceiling, floor=e.floor, B=e.B)
        elif cls == "SynChan":
            d.update(Ek=e.Ek, Gbar=e.Gbar, tau1=e.tau1, tau2=e.tau2,
                     weight=moose.element(e.path + "/sh/synapse[0]").weight)
        else:
            continue
        d["addmsg"] = [moose.element(m).value for m in moose.wildcardFind(e.path + "/addmsg#")]
        out[e.name] = d
    return out


def save_library(lib):
    out, index = {}, {}
    for name, d in lib.items():
        scalars = {k: v for k, v in d.items() if not k.startswith("gate")}
        index[name] = scalars
        for g in ("X", "Y", "Z"):
            if "gate" + g in d:
                mn, mx, A, B = d["gate" + g]
                out["lib/%s/gate%s" % (name, g)] = np.stack([A, B])
                out["lib/%s/gate%s_range" % (name, g)] = np.array([mn, mx])
    out["lib_index"] = np.array(json.dumps(index))
    return out


def run_case(moose, rd, name, spec):
    for p in ("/model", "/library"):
        if moose.exists(p):
            moose.delete(p)
    t_end = spec.pop("t_end")
    r = rd.rdesigneur(**spec)
    r.buildModel()
    h = moose.element("/model/elec/hsolve")
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
    paths = {}
    for kind, n in ((0, d.contents.n_compt), (1, d.contents.n_chan), (2, d.contents.n_pool)):
        paths[kind] = []
        for i in range(n):
            assert L.hsb_object_path(d, kind, i, buf, 512) >= 0
            paths[kind].append(buf.value.decode())
    L.hsb_free_cell_desc(d)
    lib = library(moose)
    tabs = moose.wildcardFind("/model/graphs/#[ISA=Table]")
    assert len(tabs) == 1, tabs
    moose.reinit()
    moose.start(t_end)
    vm = np.array(tabs[0].vector)
    spec["t_end"] = t_end
    stride = int(round(r.elecPlotDt / r.elecDt))
    print("%s: %d compartments, %d channels, %d pools, %d samples" % (name, m.n_compt, len(m.chan_compt),
                                                                       len(m.pool_compt), len(vm)))
    np.savez_compressed(os.path.join(HERE, "rdes_model_%s.npz" % name), spec=np.array(json.dumps(spec)),
                        vm=vm, dt=r.elecDt, stride=stride, funcDt=r.funcDt,
                        compt_paths=np.array(paths[0]), chan_paths=np.array(paths[1]),
                        pool_paths=np.array(paths[2]), **save_library(lib), **save_model(m))


def main():
    import moose
    for mod in ("matplotlib", "matplotlib.pyplot", "rdesigneur.rmoogli", "rdesigneur.moogul"):
        sys.modules.setdefault(mod, types.ModuleType(mod))
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    import rdesigneur as rd
    for name, make in CASES.items():
        run_case(moose, rd, name, make())


if __name__ == "__main__":
    main()
