"""The oracle against golden vectors produced by the reference itself.

passive_kat.json: the reference's own HinesMatrix/HSolvePassive on the nine
unit-test cells of hsolve/HinesMatrix.cpp:478-755 plus random trees with
junctions up to rank 5.  active_*.npz: full cells stepped by the reference
moose module under HSolve.  Both were written by tests/golden/make_golden.py.
The bar is bit-for-bit equality.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from loader import load_model, replay_messages
from oracle import OracleCell, OraclePassive

H = lambda v: np.array([float.fromhex(x) for x in v])


def _dense(triplets, n):
    a = np.zeros((n, n))
    for i, j, v in triplets:
        a[i, j] = float.fromhex(v)
    return a


with open(os.path.join(GOLDEN, "passive_kat.json")) as f:
    PASSIVE = json.load(f)["cells"]


@pytest.mark.parametrize("cell", PASSIVE, ids=[c["name"] for c in PASSIVE])
def test_passive_kat_bit_exact(cell):
    n = len(cell["children"])
    p = OraclePassive(cell["children"], *[H(cell[k]) for k in ("Ra", "Rm", "Cm", "Em", "V")],
                      float.fromhex(cell["dt"]))
    ref = cell["reference"]
    assert np.array_equal(p.A(), _dense(ref["A0"], n))
    for ps in ref["passes"]:
        p.update()
        assert np.array_equal(p.B(), H(ps["B"]))
        p.forward()
        assert np.array_equal(p.A(), _dense(ps["FA"], n))
        assert np.array_equal(p.B(), H(ps["FB"]))
        p.backward()
        assert np.array_equal(p.VMid(), H(ps["VMID"]))
        assert np.array_equal(p.V(), H(ps["V"]))


def run_oracle_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    m = load_model(z)
    dt = float(z["dt"])
    dts = float(z["dt_setup"]) if "dt_setup" in z.files else dt
    oc = OracleCell(m, dts)
    if "ca_advance" in z.files:
        oc.set_ca_advance(int(z["ca_advance"]))
    oc.reinit(dt)
    rec = z["rec"]
    stride, n = int(z["stride"]), int(z["nsteps"])
    vm, ca = [oc.vm()[rec]], []
    if len(m.pool_compt):
        ca.append(oc.ca()[rec])
    for _ in range(n // stride):
        oc.step(stride)
        vm.append(oc.vm()[rec])
        if len(m.pool_compt):
            ca.append(oc.ca()[rec])
    return z, oc, np.array(vm).T, (np.array(ca).T if ca else None)


@pytest.mark.parametrize("name", ["active_hh_cable", "active_branched_kca",
                                  "active_branched_caadv0"])
def test_active_golden_bit_exact(name):
    z, oc, vm, ca = run_oracle_golden(name)
    assert np.array_equal(vm, z["vm"])
    assert np.array_equal(oc.vm(), z["final_vm"])
    if ca is not None:
        assert np.array_equal(ca, z["ca"])
    assert np.array_equal(oc.spikes()[1], z["spikes"])


def test_table_grid_matches_reference():
    z = np.load(os.path.join(GOLDEN, "active_hh_cable.npz"))
    oc = OracleCell(load_model(z), float(z["dt"]))
    g = oc.table_grid()
    assert np.array_equal(g[:3], z["grid"][:3])


def test_message_destinations_and_ca_gates_bit_exact():
    """addInject, addConc (external Ca of an SK gate, V row while it is 0),
    iCa, and SK gates on the compartment's own CaConc, against the reference
    HSolve driven by StimulusTables (active_msgs.npz)."""
    z = np.load(os.path.join(GOLDEN, "active_msgs.npz"))
    m = load_model(z)
    dt = float(z["dt"])
    oc = OracleCell(m, dt)
    assert np.array_equal(oc.table_grid(), z["grid"])
    oc.reinit(dt)
    vm, ca = replay_messages(z, oc, lambda s: s.step(1))
    assert np.array_equal(vm, z["vm"])
    assert np.array_equal(ca, z["ca"])
    assert np.array_equal(oc.vm(), z["final_vm"])
