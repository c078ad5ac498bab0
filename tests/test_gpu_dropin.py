"""The FP64 drop-in HSolve on the GPU against the oracle and the reference's
golden traces.

Bars: bit-for-bit equality where no libm call is on the path (HH channels,
junctions, CaConc, SynChan, SpikeGen); for cells with an HHChannel2D (device
exp vs glibc exp) |dV| <= 1e-9 * max(|V_ref|, 1 mV) and
|dCa| <= 1e-9 * max(|Ca_ref|, CaBasal), with identical spike counts.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from loader import load_model, push_pre_reinit, replay_events, replay_messages
from moose_gb300 import _native, models
from moose_gb300.abi import HS_KIND_CHAN, HS_KIND_COMPT, HS_KIND_POOL, FIELDS, CellModel
from moose_gb300.hsolve import HSolve
from oracle import OracleCell

pytestmark = pytest.mark.gpu


def run_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    m = load_model(z)
    dt = float(z["dt"])
    h = HSolve(m, dt=float(z["dt_setup"]) if "dt_setup" in z.files else dt)
    if "ca_advance" in z.files:
        h.caAdvance = int(z["ca_advance"])
    h.target = m.seed
    rec = z["rec"]
    n, stride = int(z["nsteps"]), int(z["stride"])
    h.record(rec, stride, n // stride + 1)
    h.reinit(dt)
    cas = [h.ca()[rec]] if len(m.pool_compt) else []
    if cas:
        for _ in range(n // stride):
            h.process(stride)
            cas.append(h.ca()[rec])
    else:
        h.process(n)
    h.sync()
    return z, h, h.trace(), (np.array(cas).T if cas else None)


def test_hh_cable_golden_bit_exact():
    z, h, vm, _ = run_golden("active_hh_cable")
    assert vm.shape == z["vm"].shape
    assert np.array_equal(vm, z["vm"])
    assert np.array_equal(h.vm(), z["final_vm"])
    g, t = h.spikes()
    assert np.array_equal(t, z["spikes"])


@pytest.mark.parametrize("name", ["active_branched_kca", "active_branched_caadv0"])
def test_branched_golden_within_1e9(name):
    z, h, vm, ca = run_golden(name)
    ref = z["vm"]
    assert np.all(np.abs(vm - ref) <= 1e-9 * np.maximum(np.abs(ref), 1e-3))
    basal = 5e-5
    assert np.all(np.abs(ca - z["ca"]) <= 1e-9 * np.maximum(np.abs(z["ca"]), basal))
    assert len(h.spikes()[1]) == len(z["spikes"])


def _compare_with_oracle(m, dt, nsteps, chunk, exact=True, dt_setup=None, ca_adv=1):
    h = HSolve(m, dt=dt_setup or dt)
    h.caAdvance = ca_adv
    h.target = m.seed
    h.reinit(dt)
    oc = OracleCell(m, dt_setup or dt)
    oc.set_ca_advance(ca_adv)
    oc.reinit(dt)
    for _ in range(nsteps // chunk):
        h.process(chunk)
        oc.step(chunk)
        gv, ov = h.vm(), oc.vm()
        if exact:
            assert np.array_equal(gv, ov)
        else:
            assert np.all(np.abs(gv - ov) <= 1e-9 * np.maximum(np.abs(ov), 1e-3))
    return h, oc


@pytest.mark.parametrize("seed", range(6))
def test_random_trees_bit_exact(seed):
    """HH cells on random trees with junctions of rank up to 5."""
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(2, 400))
    parent, d, L = models.branched_morphology(rng, n, 0.6, 6)
    m = models.active_cell(parent, d, L, inject=0.6e-9, gca=15.0, gkca=0.0)
    # drop the 2-D channel so the whole path is libm-free
    for k in list(vars(m)):
        if k.startswith("c2d_"):
            setattr(m, k, getattr(m, k)[:0])
    m.gates2d = []
    m.seed = int(rng.integers(0, n))
    _compare_with_oracle(m, 25e-6, 600, 150)


def test_reference_unit_cells_bit_exact():
    """The nine unit-test cells of hsolve/HinesMatrix.cpp as passive models."""
    import json
    cells = json.load(open(os.path.join(GOLDEN, "passive_kat.json")))["cells"][:9]
    for c in cells:
        ch = c["children"]
        n = len(ch)
        parent = np.full(n, -1, np.int32)
        for p, kids in enumerate(ch):
            for k in kids:
                parent[k] = p
        i = np.arange(n, dtype=float)
        m = CellModel(parent=parent, Ra=15.0 + 3.0 * i, Rm=45.0 + 15.0 * i, Cm=500.0 + 200.0 * i * i,
                      Em=np.full(n, -0.06), initVm=-0.06 + 0.01 * i, Vm=-0.06 + 0.01 * i,
                      inject=np.zeros(n), seed=int(np.argmax(parent < 0)))
        _compare_with_oracle(m, 1.0, 20, 1)


def test_field_writes_match_oracle():
    m = models.config1_cell(n_cable=30)
    dt = 25e-6
    h, oc = _compare_with_oracle(m, dt, 200, 100)
    for obj in ((HS_KIND_COMPT, "Cm", 3, 2e-12), (HS_KIND_COMPT, "Em", 5, -0.07),
                (HS_KIND_COMPT, "Rm", 7, 3e9), (HS_KIND_COMPT, "inject", 0, 0.3e-9),
                (HS_KIND_COMPT, "Vm", 11, -0.02), (HS_KIND_CHAN, "Gbar", 4, 1e-8),
                (HS_KIND_CHAN, "X", 9, 0.5), (HS_KIND_CHAN, "modulation", 1, 1.5)):
        kind, f, i, v = obj
        h._set(kind, FIELDS[f], i, v)
        oc.set(kind, FIELDS[f], i, v)
    for _ in range(4):
        h.process(50)
        oc.step(50)
        assert np.array_equal(h.vm(), oc.vm())
    for kind, f, i in ((HS_KIND_COMPT, "Im", 4), (HS_KIND_CHAN, "Gk", 6), (HS_KIND_CHAN, "Ik", 6),
                       (HS_KIND_CHAN, "Y", 0), (HS_KIND_COMPT, "Cm", 3)):
        assert h._get(kind, FIELDS[f], i) == oc.get(kind, FIELDS[f], i)


def test_process_in_chunks_equals_one_call():
    m = models.config1_cell(n_cable=50)
    a = HSolve(m, dt=25e-6); a.target = 0; a.reinit(25e-6)
    b = HSolve(m, dt=25e-6); b.target = 0; b.reinit(25e-6)
    a.process(3000)
    for _ in range(30):
        b.process(100)
    assert np.array_equal(a.vm(), b.vm())


def test_message_destinations_golden_bit_exact():
    """addInject, addConc, iCa through the C ABI each step, and SK gates on
    the compartment's CaConc: bit-exact with the reference HSolve driven by
    StimulusTables (active_msgs.npz; no libm call on this path)."""
    z = np.load(os.path.join(GOLDEN, "active_msgs.npz"))
    m = load_model(z)
    dt = float(z["dt"])
    h = HSolve(m, dt=dt)
    h.target = m.seed
    assert [getattr(h, k) for k in ("vMin", "vMax", "vDiv", "caMin", "caMax", "caDiv")] == list(z["grid"])
    h.reinit(dt)
    vm, ca = replay_messages(z, h, lambda s: s.process(1))
    assert np.array_equal(vm, z["vm"])
    assert np.array_equal(ca, z["ca"])
    assert np.array_equal(h.vm(), z["final_vm"])


def test_add_gkek_matches_oracle():
    """HSolve::addGkEk (external channel currents) on random compartments,
    every step: bit-exact with the oracle."""
    z = np.load(os.path.join(GOLDEN, "active_msgs.npz"))
    m = load_model(z)
    h = HSolve(m, dt=25e-6)
    h.target = m.seed
    h.reinit(25e-6)
    oc = OracleCell(m, 25e-6)
    oc.reinit(25e-6)
    rng = np.random.default_rng(3)
    for k in range(300):
        for c in rng.integers(0, m.n_compt, 3):
            g, e = float(rng.uniform(0, 5e-9)), float(rng.uniform(-0.09, 0.05))
            h.add_gkek(int(c), g, e)
            oc.add_gkek(int(c), g, e)
        h.process(1)
        oc.step(1)
    assert np.array_equal(h.vm(), oc.vm())
    assert np.array_equal(h.ca(), oc.ca())


def test_runtime_events_golden():
    """hs_push_events between process calls (SimpleSynHandler::addSpike via
    Synapse::addSpike): bit-exact with the oracle on this host, and with the
    reference HSolve (active_events.npz) to 1e-12 -- the SynChan constants
    come from the host libm's exp, which may differ by an ulp between the
    machine that wrote the golden and this one.  Same spike times."""
    z = np.load(os.path.join(GOLDEN, "active_events.npz"))
    m = load_model(z)
    dt = float(z["dt"])
    h = HSolve(m, dt=dt)
    h.target = m.seed
    push_pre_reinit(z, h)
    h.reinit(dt)
    vm = replay_events(z, h, lambda s, n: s.process(n))
    oc = OracleCell(m, dt)
    push_pre_reinit(z, oc)
    oc.reinit(dt)
    ovm = replay_events(z, oc, lambda s, n: s.step(n))
    assert np.array_equal(vm, ovm)
    assert np.array_equal(h.vm(), oc.vm())
    assert np.array_equal(h.spikes()[1], oc.spikes()[1])
    ref = z["vm"]
    assert np.all(np.abs(vm - ref) <= 1e-12 * np.maximum(np.abs(ref), 1e-3))
    assert len(h.spikes()[1]) == len(z["spikes"])


def test_runtime_events_reinit_ties_and_growth():
    """Pushes of growing size (the device queue is reallocated several
    times), ties on one SynChan with different weights (summed in push
    order), events at -inf/+inf, a SynChan view's add_spike with a delay,
    and a reinit in the middle that drops the queued runtime events and
    queues the description's again: bit-exact with the oracle throughout."""
    z = np.load(os.path.join(GOLDEN, "active_events.npz"))
    m = load_model(z)
    dt = 25e-6
    ns = len(m.syn_compt)
    h = HSolve(m, dt=dt)
    h.target = m.seed
    h.reinit(dt)
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    rng = np.random.default_rng(5)
    step = 0
    for rnd in range(2):
        for chunk in range(8):
            n = 40 * 4 ** min(chunk, 4)
            k = rng.integers(0, ns, n)
            t = dt * step + rng.uniform(-2e-3, 6e-3, n)
            w = rng.uniform(0.1e-9, 1e-9, n)
            t[: n // 8] = dt * (step + 3) + 0.5 * dt          # ties with different weights
            k[: n // 8] = chunk % ns
            h.push_events(k, t, w)
            oc.push_events(k, t, w)
            if chunk == 2:
                inf = [-np.inf, np.inf]
                h.push_events([1, 2], inf, [1e-9, 1e-9])
                oc.push_events([1, 2], inf, [1e-9, 1e-9])
                h.synchan(3).add_spike(dt * step, 0.7e-9, delay=1.1e-3)
                oc.push_events([3], [dt * step + 1.1e-3], [0.7e-9])
            h.process(100)
            oc.step(100)
            step += 100
            assert np.array_equal(h.vm(), oc.vm())
        h.push_events([0, 1], [dt * (step + 5)] * 2, [5e-9, 5e-9])    # dropped by the reinit
        oc.push_events([0, 1], [dt * (step + 5)] * 2, [5e-9, 5e-9])
        h.reinit(dt)
        oc.reinit(dt)
        step = 0
    h.process(200)
    oc.step(200)
    assert np.array_equal(h.vm(), oc.vm())
    assert np.array_equal(h.spikes()[1], oc.spikes()[1])


def test_push_events_rejects_bad_input():
    z = np.load(os.path.join(GOLDEN, "active_events.npz"))
    m = load_model(z)
    h = HSolve(m, dt=25e-6)
    h.target = m.seed
    h.reinit(25e-6)
    with pytest.raises(_native.HsError):
        h.push_events([len(m.syn_compt)], [1e-3], [1e-9])
    with pytest.raises(_native.HsError):
        h.push_events([0, 1], [1e-3, float("nan")], [1e-9, 1e-9])
    h.push_events([], [], [])
    # the rejected calls queued nothing: the run equals one without pushes
    ref = HSolve(m, dt=25e-6)
    ref.target = m.seed
    ref.reinit(25e-6)
    h.process(300)
    ref.process(300)
    assert np.array_equal(h.vm(), ref.vm())


def test_field_access_between_steps_matches_oracle():
    """Zombie field reads and writes between process calls (served by the
    solver's host mirror of its device arena, writes queued until the next
    launch): reads after a step see the step's values; a read right after a
    write sees the write, also through the bulk read; the last of two writes
    to one field wins; message destinations accumulate within a step;
    CaConc setCa/setCaBasal read-modify-write; every value equal to the
    oracle's, and the run stays bit-exact with it."""
    z = np.load(os.path.join(GOLDEN, "active_msgs.npz"))
    m = load_model(z)
    dt = 25e-6
    h = HSolve(m, dt=dt)
    h.target = m.seed
    h.reinit(dt)
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    n, nch, npool = m.n_compt, len(m.chan_compt), len(m.pool_compt)
    rng = np.random.default_rng(9)
    C, CH, PL = HS_KIND_COMPT, HS_KIND_CHAN, HS_KIND_POOL

    def same(kind, f, i):
        a, b = h._get(kind, FIELDS[f], i), oc.get(kind, FIELDS[f], i)
        assert a == b, (kind, f, i, a, b)
        return a

    def put(kind, f, i, v):
        h._set(kind, FIELDS[f], i, v)
        oc.set(kind, FIELDS[f], i, v)

    for rnd in range(6):
        h.process(37)
        oc.step(37)
        for i in range(n):
            same(C, "Vm", i)
        for i in range(0, n, 5):
            same(C, "Im", i)
        for q in range(0, nch, 7):
            for f in ("Gk", "Ik", "X", "Y"):
                same(CH, f, q)
        for p in range(0, npool, 3):
            same(PL, "Ca", p)
        i = int(rng.integers(0, n))
        v = float(rng.uniform(-0.07, -0.05))
        put(C, "Vm", i, -0.03)
        put(C, "Vm", i, v)
        assert same(C, "Vm", i) == v
        assert h.vm()[i] == v
        q = int(rng.integers(0, nch))
        put(CH, "Gbar", q, float(rng.uniform(1e-9, 3e-8)))
        same(CH, "Gbar", q)
        p = int(rng.integers(0, npool))
        put(PL, "Ca", p, float(rng.uniform(6e-5, 2e-4)))
        same(PL, "Ca", p)
        put(PL, "CaBasal", p, float(rng.uniform(4e-5, 6e-5)))
        same(PL, "Ca", p)
        put(C, "inject", 0, float(rng.uniform(0.1e-9, 0.5e-9)))
        same(C, "inject", 0)
        for val in (1e-10, 2.5e-10):
            h.add_inject(0, val)
            oc.add_inject(0, val)
        h.add_ica(0, 1e-12)
        oc.add_ica(0, 1e-12)
        h.add_ica(0, 2e-12)
        oc.add_ica(0, 2e-12)
    h.process(50)
    oc.step(50)
    assert np.array_equal(h.vm(), oc.vm())
    assert np.array_equal(h.ca(), oc.ca())


@pytest.mark.parametrize("name", ["rdes_squid_axon", "rdes_current_pulse", "rdes_ball_and_stick",
                                  "rdes_periodic_syn", "rdes_squid_pulse"])
def test_rdesigneur_known_answers(name):
    """The reference's rdesigneur KATs (test_32 squid axon, test_20 current
    pulse, test_41 ball and stick, test_51 periodic synaptic input, test_30
    squid current pulse) through
    the C ABI: the soma trace recorded on the device equals
    the reference HSolve's bit for bit and passes the test's own check."""
    from test_oracle_golden import check_rdes_kat
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    m = load_model(z)
    dt = float(z["dt"])
    h = HSolve(m, dt=dt)
    h.target = m.seed
    n, stride = int(z["nsteps"]), int(z["stride"])
    h.record([0], stride, n // stride + 1)
    h.reinit(dt)
    h.process(n)
    vm = h.trace()[0]
    assert np.array_equal(vm, z["vm"])
    check_rdes_kat(z, vm)


def test_rdesigneur_minimal_model_fields():
    """tests/rdesigneur/test_1_minimalModel.py through the C ABI: the zombie
    fields right after setup equal the reference HSolve's readback exactly."""
    z = np.load(os.path.join(GOLDEN, "rdes_minimal.npz"))
    m = load_model(z)
    h = HSolve(m, dt=float(z["dt"]))
    h.target = m.seed
    got = np.array([getattr(h.compartment(0), str(k)) for k in z["kat_fields"]])
    assert np.array_equal(got, z["ref_values"])
    assert np.allclose(got, z["kat_values"], rtol=1e-12, atol=0.0)


def test_failed_record_keeps_previous_recording():
    """A rejected hs_record (a compartment outside the cell) leaves the
    recording made before it in place: the next process() writes the
    trace into live buffers and the trace equals the oracle's."""
    from moose_gb300._native import HsError
    dt = 25e-6
    m = models.config1_cell(n_cable=30, t_on=0.0, t_off=0.01)
    h = HSolve(m, dt=dt)
    h.target = 0
    h.record([0, 7], 10, 41)
    h.reinit(dt)
    with pytest.raises(HsError):
        h.record([0, 10_000], 10, 41)
    h.process(400)
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    want = [oc.vm()[[0, 7]]]
    for _ in range(40):
        oc.step(10)
        want.append(oc.vm()[[0, 7]])
    assert np.array_equal(h.trace(), np.array(want).T)
    # a new recording after process() starts its own sample count
    h.record([3], 5, 4)
    h.process(20)
    oc.step(20)
    tr = h.trace()
    assert tr.shape == (1, 4) and tr[0, -1] == oc.vm()[3]


def test_external_calcium_difshells_on_gpu():
    """tests/core/test_hsolve_externalCalcium.py on the GPU drop-in: three
    DifShells stepped on tick 1 in the reference's message order, the
    solver's IkOut into the outer shell and its concentration into the SK
    gate, 10 s at 10 us (1,000,000 steps).  Vm, the shell's Ca and SK's Gk
    every 5 ms within 1e-9 relative of the reference's (the shells'
    integration calls exp: device against glibc), and the test's own
    checks pass.  The FP64 batch steps the same cell bit-identically."""
    from moose_gb300.abi import FIELDS, HS_KIND_CHAN, HS_PREC_FP64
    from moose_gb300.batch import Batch
    from test_oracle_golden import check_ext_calcium_kat, run_ext_calcium
    z = np.load(os.path.join(GOLDEN, "ext_calcium.npz"))
    m = load_model(z)
    dt = float(z["dt"])
    h = HSolve(m, dt=dt)
    h.target = m.seed
    h.reinit(dt)
    si, ki = int(z["shell_index"]), int(z["sk_index"])
    vm, ca, sk = run_ext_calcium(h, z, lambda: h.dif()[si], lambda: h._get(HS_KIND_CHAN, FIELDS["Gk"], ki))
    for got, ref in ((vm, z["vm"]), (ca, z["shell_c"]), (sk, z["sk_gk"])):
        assert np.all(np.abs(got - ref) <= 1e-9 * np.maximum(np.abs(ref), 1e-30)), np.abs(got - ref).max()
    check_ext_calcium_kat(z, sk, ca)
    # the FP64 batch: the same arithmetic, bit-identical
    h2 = HSolve(m, dt=dt)
    h2.target = m.seed
    h2.reinit(dt)
    h2.process(20000)
    b = Batch([m], dt, HS_PREC_FP64)
    b.reinit(dt)
    b.process(20000)
    assert np.array_equal(b.vm(0), h2.vm())
    b.close()
    h.close()
    h2.close()


def test_mixed_batch_rejects_external_calcium():
    from moose_gb300._native import HsError
    from moose_gb300.abi import HS_ENOTSUP, HS_PREC_MIXED
    from moose_gb300.batch import Batch
    z = np.load(os.path.join(GOLDEN, "ext_calcium.npz"))
    with pytest.raises(HsError) as ei:
        Batch([load_model(z)], float(z["dt"]), HS_PREC_MIXED)
    assert ei.value.code == HS_ENOTSUP


def test_outgoing_values_recorded_on_device():
    """The values HSolveActive::sendValues sends each step to objects the
    solver does not own -- VmOut of compartments, IkOut = (Ek - Vm) Gk of
    HHChannels, concOut of Ca pools -- and channel Gk, recorded on the
    device every step, against the oracle read after each step (within
    1e-9 relative: the cell's K(Ca) gate calls exp)."""
    from moose_gb300.abi import HS_KIND_CHAN, HS_KIND_COMPT, HS_KIND_POOL
    z = np.load(os.path.join(GOLDEN, "active_branched_kca.npz"))
    m = load_model(z)
    dt = float(z["dt"])
    entries = ([(HS_KIND_COMPT, "Vm", i) for i in (0, 7, 31)] +
               [(HS_KIND_CHAN, "Ik", k) for k in (0, 5, 44)] + [(HS_KIND_CHAN, "Gk", k) for k in (2, 44)] +
               [(HS_KIND_POOL, "Ca", p) for p in (0, 9)])
    n = 300
    h = HSolve(m, dt=dt)
    h.target = m.seed
    h.record_values(entries, 1, n + 1)
    h.reinit(dt)
    h.process(n)
    got = h.trace()
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    rows = []
    for s in range(n):
        oc.step(1)
        rows.append([oc.get(k, FIELDS[f], i) if k != HS_KIND_POOL else oc.ca()[i] for k, f, i in entries])
    want = np.array(rows).T
    assert got.shape == (len(entries), n + 1)
    assert np.all(np.abs(got[:, 1:] - want) <= 1e-9 * np.maximum(np.abs(want), 1e-15))
    # Ik is what the reference sends: (Ek - Vm) Gk of the channel's compartment
    assert np.any(np.abs(got[3:6, 1:]) > 0)
    with pytest.raises(_native.HsError):
        h.record_values([(HS_KIND_POOL, "Vm", 0)], 1, 4)
    h.close()
