"""moose_gb300.inputs (TimeTable-driven SynChans) against the reference
HSolve with real TimeTables (tests/golden/make_golden_timetable.py): the
oracle, given the queued events the helper derives, reproduces the
reference's soma trace and final Vm bit for bit -- including entries sent
one per tick (bursts closer than a tick), entries between steps, synapse
delays and a table on tick 0 (before the handler: an entry can reach the
synapse in the step it is sent in).  PulseGens and StimulusTables into
injectMsg likewise (tests/golden/make_golden_pulsegen.py)."""
import os

import numpy as np

from conftest import GOLDEN
from loader import load_model
from moose_gb300 import inputs
from oracle import OracleCell

Z = np.load(os.path.join(GOLDEN, "timetable_golden.npz"))


def _model():
    m = load_model(Z)
    dt, n, stride = float(Z["dt"]), int(Z["nsteps"]), int(Z["stride"])
    tables = {k: (Z["tt%d_times" % k], float(Z["tt%d_delay" % k]), float(Z["tt%d_weight" % k]))
              for k in range(len(m.syn_compt))}
    import sys
    sys.path.insert(0, GOLDEN)
    from make_golden_timetable import EARLY
    m = inputs.add_timetables(m, {k: v for k, v in tables.items() if k not in EARLY}, dt, n, stride)
    m = inputs.add_timetables(m, {k: v for k, v in tables.items() if k in EARLY}, dt, n, 1, before_handler=EARLY)
    return m, dt, n, stride


def test_timetable_events_reproduce_the_reference_run():
    m, dt, n, stride = _model()
    assert len(m.ev_syn) > 40
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    vm = [oc.vm()[0]]
    for _ in range(n // stride):
        oc.step(stride)
        vm.append(oc.vm()[0])
    assert np.array_equal(np.array(vm), Z["vm"])
    assert np.array_equal(oc.vm(), Z["final_vm"])


def test_one_entry_per_tick_and_delivery_step():
    dt = 25e-6
    # three entries inside one tick of 4 steps go out on three ticks
    ev = inputs.timetable_events([1e-3, 1.01e-3, 1.02e-3], dt, 200, stride=4)
    assert np.array_equal(ev, [dt * 41, dt * 45, dt * 49])
    # a delay that reaches past the next step keeps the event's own time
    ev = inputs.timetable_events([1e-3], dt, 200, stride=4, delay=1e-3)
    assert ev[0] == 1e-3 + 1e-3
    # an entry the run never reaches is not sent
    assert len(inputs.timetable_events([1.0], dt, 200)) == 0


P = np.load(os.path.join(GOLDEN, "pulsegen_golden.npz"))


def test_pulsegens_reproduce_the_reference_run():
    """Three free-running PulseGens into injectMsg (one with a base level
    that its reinit also sends, one on a tick of three steps into a
    compartment with its own inject field, one on a tick after the
    solver's) and two StimulusTables (one
    looping at the clock time, one advancing by its own step): the oracle
    with the derived inject schedule equals the reference's traces (every
    4 steps) and final Vm bit for bit."""
    import sys
    sys.path.insert(0, GOLDEN)
    from make_golden_pulsegen import PULSES, STIMTABLES
    m = load_model(P)
    dt, n = float(P["dt"]), int(P["nsteps"])
    for c, (level, width, delay, base, tick, k) in PULSES.items():
        inputs.add_pulsegen(m, c, inputs.PulseGen(level, width, delay, base), dt, n, stride=k,
                            after_solver=tick > 6)
    for c, (vec, start, stop, step, loop, loop_t) in STIMTABLES.items():
        inputs.add_injector(m, c, inputs.StimulusTable(vec, start, stop, step, loop, loop_t), dt, n)
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    rec = P["rec"]
    vm = [oc.vm()[rec]]
    for _ in range(n // 4):
        oc.step(4)
        vm.append(oc.vm()[rec])
    assert np.array_equal(np.array(vm).T, P["vm"])
    assert np.array_equal(oc.vm(), P["final_vm"])


def test_pulsegen_output_keeps_the_reference_rules():
    pg = inputs.PulseGen([1.0, 2.0], [0.01, 0.02], [0.005, 0.01], baseLevel=0.5)
    assert pg.reinit() == 0.5
    # period: w0 + d0, plus d1 + w1 - w0 = 0.035; the second pulse's delay
    # counts from the first pulse's start
    assert pg.process(0.001) == 0.5          # before the first pulse
    assert pg.process(0.006) == 1.0          # first pulse
    assert pg.process(0.016) == 2.0          # second pulse
    assert pg.process(0.036) == 0.5          # the next period
