"""moose_gb300.stats (Stats, SpikeStats) against the reference's own Stats
and SpikeStats objects run beside the reference HSolve
(tests/golden/make_golden_stats.py): the oracle steps the same cell
(bit-exact with the reference HSolve), and the statistics of its soma Vm
sampled on the Stats tick and of its spike times on the SpikeStats tick
equal the reference objects' fields bit for bit."""
import os

import numpy as np

from conftest import GOLDEN
from loader import load_model
from moose_gb300 import stats
from oracle import OracleCell

Z = np.load(os.path.join(GOLDEN, "stats_golden.npz"))
FIELDS = ("mean", "sdev", "sum", "num", "wmean", "wsdev", "wsum", "wnum")


def _run():
    m = load_model(Z)
    dt, n, k = float(Z["dt"]), int(Z["nsteps"]), int(Z["st_stride"])
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    vm = []
    for _ in range(n // k):
        oc.step(k)
        vm.append(oc.vm()[0])
    return oc.spikes()[1], np.array(vm)


def test_oracle_spikes_are_the_reference_spikes():
    spikes, _ = _run()
    assert np.array_equal(spikes, Z["spikes"])


def test_stats_and_spike_stats_match_the_reference_objects():
    spikes, vm = _run()
    dt, n = float(Z["dt"]), int(Z["nsteps"])
    st = stats.stats_of_samples(vm, int(Z["st_window"]))
    ss = stats.spike_stats_of_times(spikes, dt, int(Z["ss_stride"]), n, int(Z["ss_window"]))
    for f in FIELDS:
        assert getattr(st, f) == Z["st_" + f], ("Stats", f, getattr(st, f), Z["st_" + f])
        assert getattr(ss, f) == Z["ss_" + f], ("SpikeStats", f, getattr(ss, f), Z["ss_" + f])


def test_spike_stats_vm_input_counts_upward_crossings():
    s = stats.SpikeStats(threshold=0.0)
    for v in (-0.07, 0.01, 0.02, -0.01, 0.03, -0.06):
        s.vm(v)
    assert s.num_spikes == 2
    s.process(1e-3)
    assert s.sum == 2000.0 and s.num == 1
