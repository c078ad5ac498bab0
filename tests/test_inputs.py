"""moose_gb300.inputs (TimeTable-driven SynChans) against the reference
HSolve with real TimeTables (tests/golden/make_golden_timetable.py): the
oracle, given the queued events the helper derives, reproduces the
reference's soma trace and final Vm bit for bit -- including entries sent
one per tick (bursts closer than a tick), entries between steps and
synapse delays."""
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
    return inputs.add_timetables(m, tables, dt, n, stride), dt, n, stride


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
