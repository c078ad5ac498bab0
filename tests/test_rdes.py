"""The rdesigneur loader (moose_gb300.rdes) against models the reference's
own rdesigneur built (tests/golden/make_golden_rdes_model.py): the test_41
ball and stick, the test_20 passive soma under a pulse, and a branchedCell
with passive and channel distributions over p, g, L, dia, maxP (exp, H,
?:, ^), a Ca channel feeding a CaConc and a K_AHP reading it, and one
with make_glu SynChans distributed over the dendrites.

From the same rdesigneur arguments and the reference's /library prototypes,
the loader's model equals the reference HSolve's description (from the
MOOSE-side binding) object by object: every compartment's Ra, Rm, Cm, Em,
initVm, each compartment's channels in message order with Gbar and Ek,
each pool's B, tau and CaBasal, the Ca links; and the oracle stepping the
loader's model, with the stimulus schedule it derives from the stimulus
expression, reproduces the reference's soma plot bit for bit."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from loader import load_model
from moose_gb300 import genesis
from moose_gb300.rdes import Rdesigneur
from oracle import OracleCell

CASES = ["ball_and_stick", "soma_pulse", "branched_distrib", "glu_distrib"]


def _z(name):
    return np.load(os.path.join(GOLDEN, "rdes_model_%s.npz" % name))


def library_from(z):
    """The reference's /library prototypes as genesis prototype objects."""
    index = json.loads(str(z["lib_index"]))
    lib = {}
    for name, d in index.items():
        if d["class"].endswith("CaConc"):
            p = genesis.CaConcProto(tau=d["tau"], CaBasal=d["CaBasal"], thick=d["thick"],
                                    diameter=d["diameter"], length=d["length"], ceiling=d["ceiling"],
                                    floor=d["floor"], addmsg=d["addmsg"])
        elif d["class"] == "SynChan":
            p = genesis.SynChanProto(Ek=d["Ek"], tau1=d["tau1"], tau2=d["tau2"], weight=d["weight"],
                                     addmsg=d["addmsg"])
        else:
            gate = {}
            for g in ("X", "Y", "Z"):
                key = "lib/%s/gate%s" % (name, g)
                if key in z.files:
                    mn, mx = z[key + "_range"]
                    gate[g] = (float(mn), float(mx), z[key][0], z[key][1])
            p = genesis.HHChannelProto(Ek=d["Ek"], Xpower=d["Xpower"], Ypower=d["Ypower"], Zpower=d["Zpower"],
                                       xgate=gate.get("X"), ygate=gate.get("Y"), zgate=gate.get("Z"),
                                       instant=d["instant"], useConcentration=d["useConcentration"],
                                       addmsg=d["addmsg"])
        p.Gbar = d.get("Gbar", 0.0)
        lib[name] = p
    return lib


def build(z):
    spec = json.loads(str(z["spec"]))
    r = Rdesigneur(cellProto=spec.get("cellProto", []), library=library_from(z),
                   passiveDistrib=spec.get("passiveDistrib", []), chanDistrib=spec.get("chanDistrib", []),
                   stimList=spec.get("stimList", []), elecDt=float(z["dt"]), funcDt=float(z["funcDt"]))
    return r.build_model(spec["t_end"])


def _leaf(path):
    return path.split("/")[-1].split("[")[0]


@pytest.mark.parametrize("name", CASES)
def test_loader_model_equals_reference_description(name):
    z = _z(name)
    m = build(z)
    ref = load_model(z)
    names = m.meta["names"]
    mine = {n: i for i, n in enumerate(names)}
    ref_names = [_leaf(p) for p in z["compt_paths"]]
    assert sorted(ref_names) == sorted(names)
    where = np.array([mine[n] for n in ref_names])          # reference index -> loader index
    for f in ("Ra", "Rm", "Cm", "Em", "initVm"):
        assert np.array_equal(getattr(m, f)[where], getattr(ref, f)), f
    # channels of each compartment, in message order
    chan_names = [_leaf(p) for p in z["chan_paths"]]
    for r_i, i in enumerate(where):
        got = [k for k in range(len(m.chan_compt)) if m.chan_compt[k] == i]
        exp = [k for k in range(len(ref.chan_compt)) if ref.chan_compt[k] == r_i]
        assert [m.meta["chan_name"][k] for k in got] == [chan_names[k] for k in exp], names[i]
        assert np.array_equal(m.chan_Gbar[got], ref.chan_Gbar[exp]), names[i]
        assert np.array_equal(m.chan_Ek[got], ref.chan_Ek[exp]), names[i]
        for f in ("chan_ca_target", "chan_ca_depend"):
            a, b = getattr(m, f)[got], getattr(ref, f)[exp]
            assert np.array_equal(a >= 0, b >= 0), (names[i], f)
            assert np.array_equal(m.pool_compt[a[a >= 0]], where[ref.pool_compt[b[b >= 0]]]), (names[i], f)
    # SynChans of each compartment, in order
    assert len(m.syn_compt) == len(ref.syn_compt)
    for r_i, i in enumerate(where):
        got = np.nonzero(m.syn_compt == i)[0]
        exp = np.nonzero(ref.syn_compt == r_i)[0]
        for f in ("syn_Gbar", "syn_Ek", "syn_tau1", "syn_tau2"):
            assert np.array_equal(getattr(m, f)[got], getattr(ref, f)[exp]), (names[i], f)
    # pools
    assert len(m.pool_compt) == len(ref.pool_compt)
    for r_k in range(len(ref.pool_compt)):
        k = int(np.nonzero(m.pool_compt == where[ref.pool_compt[r_k]])[0][0])
        for f in ("pool_B", "pool_tau", "pool_CaBasal", "pool_ceiling", "pool_floor"):
            assert getattr(m, f)[k] == getattr(ref, f)[r_k], (f, r_k)
    assert names[m.seed] == ref_names[ref.seed] or names[m.seed] == "soma"


@pytest.mark.parametrize("name", CASES)
def test_loader_model_reproduces_reference_trace(name):
    z = _z(name)
    m = build(z)
    dt, stride = float(z["dt"]), int(z["stride"])
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    soma = m.seed
    vm = [oc.vm()[soma]]
    for _ in range(len(z["vm"]) - 1):
        oc.step(stride)
        vm.append(oc.vm()[soma])
    assert np.array_equal(np.array(vm), z["vm"])


def test_expression_numbers_follow_exprtk():
    """exprtk reads a literal digit by digit (not correctly rounded) and
    turns integer powers into fixed product chains."""
    from moose_gb300.exprtk_eval import Expression, exprtk_number
    # 0.1 + 0.2-style fractions are built as digits / 10^k
    assert exprtk_number("1.2e-6") == (1.0 + 2.0 / 10.0) / 1e6
    assert exprtk_number("0.33333333") == 33333333.0 / 1e8
    x = 1.1
    assert Expression("x^3")(x=x) == x * x * x
    assert Expression("x^4")(x=x) == (x * x) * (x * x)
    assert Expression("x^-2")(x=x) == 1.0 / (x * x)
    assert Expression("x^0.5")(x=x) == x ** 0.5
    assert Expression("(t>0.01 && t<0.05) * 1e-9")(t=0.02) == 1e-9
    assert Expression("dia > 2e-6 ? 300 : 150")(dia=1e-6) == 150.0
    assert Expression("H(g - 1) + not (g > 5)")(g=2.0) == 2.0
    with pytest.raises(ValueError):
        Expression("2^3^2")
    with pytest.raises(ValueError):
        Expression("unknown(3)")


def test_rejected_arguments():
    with pytest.raises(ValueError):
        Rdesigneur(cellProto=[["spineProto", "x"]]).build_model()
    with pytest.raises(ValueError):
        Rdesigneur(chanDistrib=[["Na", "soma", "Gbar", "1200"]]).build_model()     # not in the library
    with pytest.raises(ValueError):
        Rdesigneur(chanDistrib=[["Na", "soma", "Gbar"]], library={"Na": None}).build_model()
    with pytest.raises(ValueError):
        Rdesigneur(stimList=[["soma", "1", ".", "randsyn", "5"]]).build_model()


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_loader_model_on_gpu_dropin(name):
    from moose_gb300.hsolve import HSolve
    z = _z(name)
    m = build(z)
    dt, stride = float(z["dt"]), int(z["stride"])
    h = HSolve(m, dt=dt)
    h.target = m.seed
    h.record([m.seed], stride, len(z["vm"]))
    h.reinit(dt)
    h.process(stride * (len(z["vm"]) - 1))
    h.sync()
    assert np.array_equal(h.trace()[0], z["vm"])
    h.close()
