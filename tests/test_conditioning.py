"""The oracle's conditioning probe (FP32 gate increments accumulated in FP64,
the gating precision of the mixed-precision solver), used to tell an
ill-conditioned cell from a solver defect when the mixed batch leaves the
0.1 mV / 0.05 ms bar over the synaptic workload's full second.

Off by default (the golden tests run with it off and stay bit-exact).  Cell
861 of the 4,096-cell synaptic workload (136 compartments) is
ill-conditioned: over 1 s the probe alone moves its soma by about 2 mV
(20 times the 0.1 mV bar; the larger cell 2528 moves by tens of mV and
changes its spike count).  Cell 158 is well conditioned: the probe moves it
by microvolts.  CPU only."""
import numpy as np

from moose_gb300 import models
from oracle import OracleCell

DT = 25e-6
N = 40000


def _soma(m, probe, every=20):
    o = OracleCell(m, DT)
    o.set_f32_gate_increments(probe)
    o.reinit(DT)
    v = [o.vm()[0]]
    for _ in range(N // every):
        o.step(every)
        v.append(o.vm()[0])
    return np.array(v), np.sort(o.spikes()[1])


def _cell(i):
    sizes, _, _ = models.population_sizes(4, 1, 4096)
    return models.make_cell(4, 1, i, t_end=N * DT + 0.01, sizes=sizes)


def test_probe_separates_ill_from_well_conditioned_cells():
    ill = _cell(861)
    a, ta = _soma(ill, False)
    b, tb = _soma(ill, True)
    assert np.abs(a - b).max() > 1e-3 or len(ta) != len(tb)
    well = _cell(158)
    c, tc = _soma(well, False)
    d, td = _soma(well, True)
    assert np.abs(c - d).max() < 1e-5
    assert np.array_equal(tc, td)
