"""SWC morphologies (moose_gb300.swc) on the GPU.

Passive cells exactly as the reference's loadModel builds them: the FP64
drop-in HSolve against the reference HSolve's traces in
tests/golden/swc_golden.npz, bit for bit.  The same morphologies with the
workload's channels (HH Na/K, Ca(HVA) into a CaConc, K(Ca) HHChannel2D,
SynChans): the FP64 drop-in within |dV| <= 1e-9 max(|V|, 1 mV) of the oracle
(the K(Ca) gate calls exp) with identical spike counts, and the mixed batch
within 0.1 mV and 0.05 ms of the oracle.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from moose_gb300 import models, swc
from moose_gb300.abi import HS_PREC_MIXED
from moose_gb300.batch import Batch
from moose_gb300.hsolve import HSolve
from oracle import OracleCell

pytestmark = pytest.mark.gpu

Z = np.load(os.path.join(GOLDEN, "swc_golden.npz"))
VALID = sorted({k.split("/")[0] for k in Z.files if "/" in k and not k.startswith("invalid")})
DT = 25e-6


def path(name):
    return os.path.join(GOLDEN, "swc", name + ".swc")


@pytest.mark.parametrize("name", VALID)
def test_passive_swc_dropin_bit_exact_with_reference(name):
    m = swc.load_swc(path(name))
    m.inject[0] = float(Z["inject"])
    dt, stride, n = float(Z["dt"]), int(Z["stride"]), int(Z["nsteps"])
    h = HSolve(m, dt=dt)
    h.target = m.seed
    h.record([0, m.n_compt - 1], stride, n // stride + 1)
    h.reinit(dt)
    h.process(n)
    h.sync()
    assert np.array_equal(h.trace(), Z[name + "/trace"])
    assert np.array_equal(h.vm(), Z[name + "/final_vm"])


def active_cells():
    kA, kB = models.kca_2d_tables(vdivs=300, cadivs=300)
    return [swc.active_swc_cell(path(nm), inject=0.6e-9, kca_tables=(kA, kB), t_end=0.1, n_syn=20,
                                syn_rate=40.0, rng=np.random.default_rng(i)) for i, nm in enumerate(VALID)]


def test_active_swc_dropin_within_1e9_of_oracle():
    for m in active_cells():
        h = HSolve(m, dt=DT)
        h.target = m.seed
        h.reinit(DT)
        oc = OracleCell(m, DT)
        oc.reinit(DT)
        for _ in range(4):
            h.process(200)
            oc.step(200)
            ov = oc.vm()
            assert np.all(np.abs(h.vm() - ov) <= 1e-9 * np.maximum(np.abs(ov), 1e-3))
        assert len(h.spikes()[1]) == len(oc.spikes()[1])


def test_active_swc_mixed_batch_within_tolerance():
    cells = active_cells()
    b = Batch(cells, DT, HS_PREC_MIXED, steps_per_launch=100)
    b.reinit(DT)
    oracles = []
    for m in cells:
        oc = OracleCell(m, DT)
        oc.reinit(DT)
        oracles.append(oc)
    worst = 0.0
    for _ in range(20):
        b.process(200)
        for i, oc in enumerate(oracles):
            oc.step(200)
            worst = max(worst, float(np.abs(b.vm(i) - oc.vm()).max()))
    assert worst <= 1e-4, "max |dVm| = %g V" % worst
    cell_ids, gens, t = b.spikes()
    spiked = 0
    for i, oc in enumerate(oracles):
        ref = oc.spikes()[1]
        got = np.sort(t[cell_ids == i])
        assert len(got) == len(ref), "cell %d spike count %d vs %d" % (i, len(got), len(ref))
        if len(ref):
            spiked += 1
            assert np.abs(got - ref).max() <= 5e-5
    assert spiked > 0
