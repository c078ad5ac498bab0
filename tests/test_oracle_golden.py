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
from loader import load_model, push_pre_reinit, replay_events, replay_messages
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


def test_runtime_events_bit_exact():
    """Synaptic events pushed between process calls (SimpleSynHandler::addSpike
    via Synapse::addSpike with its delay): late events, events on a step's
    clock time, two synapses of one handler, events pushed before reinit
    (dropped), against the reference HSolve (active_events.npz)."""
    z = np.load(os.path.join(GOLDEN, "active_events.npz"))
    m = load_model(z)
    dt = float(z["dt"])
    oc = OracleCell(m, dt)
    push_pre_reinit(z, oc)
    oc.reinit(dt)
    vm = replay_events(z, oc, lambda s, n: s.step(n))
    assert np.array_equal(vm, z["vm"])
    assert np.array_equal(oc.vm(), z["final_vm"])
    assert np.array_equal(oc.spikes()[1], z["spikes"])


def test_runtime_events_change_the_trace():
    """The pushed events matter: without them the trace differs from the
    golden (so the bit-exact match above is not vacuous)."""
    z = np.load(os.path.join(GOLDEN, "active_events.npz"))
    m = load_model(z)
    dt = float(z["dt"])
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    oc.step(int(z["nsteps"]))
    assert not np.array_equal(oc.vm(), z["final_vm"])


def test_oracle_push_event_rejects_bad_input():
    z = np.load(os.path.join(GOLDEN, "active_events.npz"))
    oc = OracleCell(load_model(z), float(z["dt"]))
    with pytest.raises(IndexError):
        oc.push_events([len(z["model_syn_compt"])], [0.0], [1e-9])
    with pytest.raises(IndexError):
        oc.push_events([0], [float("nan")], [1e-9])


def test_runtime_events_golden_pins_reinit_drop_and_clock_time():
    """Two mistakes planted in how the oracle is driven both break the match:
    keeping the events pushed before reinit, and events on a step's clock
    time arriving one ulp later (one step late).  So the golden pins
    SimpleSynHandler::vReinit's drop and the `time <= currTime` test."""
    z = np.load(os.path.join(GOLDEN, "active_events.npz"))
    m = load_model(z)
    dt = float(z["dt"])
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    push_pre_reinit(z, oc)
    assert not np.array_equal(replay_events(z, oc, lambda s, n: s.step(n)), z["vm"])
    zz = dict(z)
    pt = zz["push_time"].copy()
    on_clock = pt == dt * np.round(pt / dt)
    assert on_clock.sum() >= 50
    pt[on_clock] = np.nextafter(pt[on_clock], np.inf)
    zz["push_time"] = pt
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    assert not np.array_equal(replay_events(zz, oc, lambda s, n: s.step(n)), z["vm"])


def _soma_trace(solver, z, advance):
    stride, n = int(z["stride"]), int(z["nsteps"])
    vm = [solver.vm()[0]]
    for _ in range(n // stride):
        advance(solver, stride)
        vm.append(solver.vm()[0])
    return np.array(vm)


def check_rdes_kat(z, vm):
    """The reference test's own assertion on the soma trace."""
    if "kat_atol" in z.files:        # tests/rdesigneur/test_41_ballAndStick.py (3 decimals)
        assert np.allclose(vm[::int(z["kat_every"])], z["kat_samples"], rtol=0.0, atol=float(z["kat_atol"]) + 1e-12)
    elif "kat_samples" in z.files:   # tests/rdesigneur/test_32_squid_axon_propgn.py
        assert np.allclose(vm[::int(z["kat_every"])], z["kat_samples"])
    elif "kat_head" in z.files:      # tests/rdesigneur/test_30_squid_currentPulse.py (8 decimals)
        h, t = z["kat_head"], z["kat_tail"]
        assert np.allclose(vm[:len(h)], h, rtol=0.0, atol=5e-9 + 1e-15)
        assert np.allclose(vm[-len(t):], t, rtol=0.0, atol=5e-9 + 1e-15)
        assert np.allclose([z["kat_mean"], z["kat_std"]], [vm.mean(), vm.std()])
    elif "kat_rtol" in z.files:      # tests/rdesigneur/test_51_periodic_syn_input.py
        assert np.allclose([z["kat_mean"], z["kat_std"]], [vm.mean(), vm.std()], rtol=float(z["kat_rtol"]))
    else:                            # tests/rdesigneur/test_20_currentPulse.py
        hist, edges = np.histogram(vm)
        assert np.allclose(vm.mean(), z["kat_mean"]) and np.allclose(vm.std(), z["kat_std"])
        assert np.allclose(hist, z["kat_hist"]) and np.allclose(edges, z["kat_edges"])


@pytest.mark.parametrize("name", ["rdes_squid_axon", "rdes_current_pulse", "rdes_ball_and_stick",
                                  "rdes_periodic_syn", "rdes_squid_pulse"])
def test_rdesigneur_known_answers(name):
    """The reference's rdesigneur KATs (test_32 squid axon: 201
    compartments, Na/K gates on different voltage grids merged by the
    solver; test_20 passive soma under a current pulse; test_41 ball and
    stick with per-region channel densities; test_51 a SynChan driven at
    50 Hz through Synapse::addSpike; test_30 an HH squid soma under a
    current pulse), assembled and run
    by the reference HSolve (make_golden_rdes.py): the oracle's soma trace
    equals the reference's bit for bit and passes the test's own check."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    m = load_model(z)
    dt = float(z["dt"])
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    vm = _soma_trace(oc, z, lambda s, n: s.step(n))
    assert np.array_equal(vm, z["vm"])
    check_rdes_kat(z, vm)


def test_rdesigneur_minimal_model_fields():
    """tests/rdesigneur/test_1_minimalModel.py: the passive soma's zombie
    fields right after setup (Cm, Em, Im, Ra, Rm, Vm, initVm, inject) equal
    the reference HSolve's readback exactly and the doctest's printed
    values to their printed precision."""
    from moose_gb300.abi import FIELDS, HS_KIND_COMPT
    z = np.load(os.path.join(GOLDEN, "rdes_minimal.npz"))
    oc = OracleCell(load_model(z), float(z["dt"]))
    got = np.array([oc.get(HS_KIND_COMPT, FIELDS[str(k)], 0) for k in z["kat_fields"]])
    assert np.array_equal(got, z["ref_values"])
    assert np.allclose(got, z["kat_values"], rtol=1e-12, atol=0.0)


def check_ext_calcium_kat(z, sk, ca):
    """tests/core/test_hsolve_externalCalcium.py's own assertions: min, max,
    mean and std of the SK conductance and of the outer shell's Ca (np.allclose
    defaults), and the counts of samples below/above its thresholds."""
    stat = lambda v: [np.min(v), np.max(v), np.mean(v), np.std(v)]
    assert np.allclose(stat(sk), z["kat_sk"])
    assert np.allclose(stat(ca), z["kat_ca"])
    assert len(np.where(sk < 1e-19)[0]) == 2001
    assert len(np.where(ca > 50e-6)[0]) == 2000


def run_ext_calcium(solver, z, read_shell, read_sk):
    stride, n = int(z["stride"]), int(z["nsteps"])
    vm, ca, sk = [solver.vm()[0]], [read_shell()], [read_sk()]
    for _ in range(n // stride):
        solver.step(stride) if hasattr(solver, "step") else solver.process(stride)
        vm.append(solver.vm()[0])
        ca.append(read_shell())
        sk.append(read_sk())
    return np.array(vm), np.array(ca), np.array(sk)


def test_external_calcium_difshells_bit_exact():
    """tests/core/test_hsolve_externalCalcium.py: a soma whose CaL12 current
    (the solver's IkOut) flows into the outer of three DifShells and whose SK
    gate reads that shell (concentrationOut -> HSolve::addConc), 10 s at
    10 us (ext_calcium.npz, made by the reference itself, its model described
    by the MOOSE-side binding): Vm, the shell's Ca and SK's Gk every 5 ms
    equal the reference's bit for bit, and the test's own checks pass."""
    from moose_gb300.abi import FIELDS, HS_KIND_CHAN
    z = np.load(os.path.join(GOLDEN, "ext_calcium.npz"))
    m = load_model(z)
    dt = float(z["dt"])
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    si, ki = int(z["shell_index"]), int(z["sk_index"])
    vm, ca, sk = run_ext_calcium(oc, z, lambda: oc.dif()[si], lambda: oc.get(HS_KIND_CHAN, FIELDS["Gk"], ki))
    assert np.array_equal(vm, z["vm"])
    assert np.array_equal(ca, z["shell_c"])
    assert np.array_equal(sk, z["sk_gk"])
    check_ext_calcium_kat(z, sk, ca)


def test_external_calcium_drives_the_cell():
    """The shells matter: with the IkOut influx removed the shell stays at
    its equilibrium and the trace differs (the match above is not vacuous)."""
    z = np.load(os.path.join(GOLDEN, "ext_calcium.npz"))
    m = load_model(z)
    keep = m.dmsg_kind != 6          # HS_DMSG_IK
    m.dmsg_kind, m.dmsg_src, m.dmsg_dst = m.dmsg_kind[keep], m.dmsg_src[keep], m.dmsg_dst[keep]
    dt = float(z["dt"])
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    oc.step(200000)
    assert oc.dif()[int(z["shell_index"])] == 5e-5
