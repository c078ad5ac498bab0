"""GENESIS .p cells (moose_gb300.genesis) on the GPU: the FP64 drop-in
against the oracle and the reference HSolve's traces (genesis_golden.npz),
bit-exact where no libm call is involved, else within
|dV| <= 1e-9 max(|V|, 1 mV) with the same spike times; the mixed batch
within 0.1 mV and 0.05 ms of the oracle.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN
from moose_gb300 import genesis, models
from moose_gb300.abi import HS_PREC_MIXED
from moose_gb300.batch import Batch
from moose_gb300.hsolve import HSolve
from oracle import OracleCell

sys.path.insert(0, GOLDEN)
from make_golden_genesis import library  # noqa: E402

pytestmark = pytest.mark.gpu

Z = np.load(os.path.join(GOLDEN, "genesis_golden.npz"))
FILES = sorted({k.split("/")[0] for k in Z.files if "/" in k})
LIB = library(Z)


def path(name):
    return os.path.join(GOLDEN, "genesis", name + ".p")


@pytest.mark.parametrize("name", FILES)
def test_dropin_matches_reference_hsolve(name):
    """Against the oracle on the same loaded model: bit-exact unless the cell
    has a K(Ca) gate (exp).  Against the reference's traces: bit-exact when
    neither the cell (K(Ca)) nor the loader (polar coordinates: sin/cos of
    this machine's libm) calls libm, else within 1e-9.  The synaptic events
    the reference queued are the model's queued events."""
    m = genesis.load_p(path(name), LIB)
    if name + "/ev_syn" in Z.files:
        m.ev_syn, m.ev_time, m.ev_weight = Z[name + "/ev_syn"], Z[name + "/ev_time"], Z[name + "/ev_weight"]
    m.inject[0] = float(Z["inject"])
    dt, stride, n = float(Z["dt"]), int(Z["stride"]), int(Z["nsteps"])
    rec = Z[name + "/rec"]
    h = HSolve(m, dt=dt)
    h.target = m.seed
    h.record(rec, stride, n // stride + 1)
    h.reinit(dt)
    h.process(n)
    h.sync()
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    oc.step(n)
    exp_free = len(m.c2d_compt) == 0
    with open(path(name)) as f:
        libm_free = exp_free and "*polar" not in f.read()
    close = lambda a, r: np.all(np.abs(a - r) <= 1e-9 * np.maximum(np.abs(r), 1e-3))
    if exp_free:
        assert np.array_equal(h.vm(), oc.vm())
    else:
        assert close(h.vm(), oc.vm())
    ref = Z[name + "/vm"]
    if libm_free:
        assert np.array_equal(h.trace(), ref)
        assert np.array_equal(h.vm(), Z[name + "/final_vm"])
        assert np.array_equal(h.spikes()[1], Z[name + "/spikes"])
    else:
        assert close(h.trace(), ref)
        assert np.all(np.abs(h.spikes()[1] - Z[name + "/spikes"]) <= 1e-12)
    assert len(h.spikes()[1]) == len(Z[name + "/spikes"])


def _run(cells, n=4000):
    b = Batch(cells, 25e-6, HS_PREC_MIXED, steps_per_launch=100)
    b.reinit(25e-6)
    b.process(n)
    return b


def test_mixed_batch_of_different_channel_sets():
    """Cells with different channel libraries in one mixed batch (their rate
    tables merged into one): each within 0.1 mV / 0.05 ms of the oracle, and
    bit-identical to the same cell in a batch of its own channel set."""
    cells = []
    for k, name in enumerate(("relative_cartesian", "relative_cartesian", "absolute_polar", "spherical_soma")):
        m = genesis.load_p(path(name), LIB)
        m.inject[0] = float(Z["inject"]) * (1.0 + 0.5 * k)
        cells.append(m)
    kA, kB = models.kca_2d_tables(vdivs=300, cadivs=300)
    rng = np.random.default_rng(5)
    parent, d, L = models.branched_morphology(rng, 150, 0.5, 4)
    cells.append(models.active_cell(parent, d, L, inject=0.6e-9, kca_tables=(kA, kB), t_end=0.1))
    cells.append(models.config1_cell(n_cable=60, inject=0.4e-9))
    b = Batch(cells, 25e-6, HS_PREC_MIXED, steps_per_launch=100)
    b.reinit(25e-6)
    oracles = []
    for m in cells:
        oc = OracleCell(m, 25e-6)
        oc.reinit(25e-6)
        oracles.append(oc)
    worst = 0.0
    for _ in range(20):
        b.process(200)
        for i, oc in enumerate(oracles):
            oc.step(200)
            worst = max(worst, float(np.abs(b.vm(i) - oc.vm()).max()))
    assert worst <= 1e-4, "max |dVm| = %g V" % worst
    cell_ids, gens, t = b.spikes()
    for i, oc in enumerate(oracles):
        ref = oc.spikes()[1]
        got = np.sort(t[cell_ids == i])
        assert len(got) == len(ref), "cell %d spike count %d vs %d" % (i, len(got), len(ref))
        if len(ref):
            assert np.abs(got - ref).max() <= 5e-5
    alone = _run(cells[:2])
    hh = _run(cells[2:4])
    for i in range(2):
        assert np.array_equal(alone.vm(i), b.vm(i))
        assert np.array_equal(hh.vm(i), b.vm(2 + i))


def test_mixed_batch_rejects_different_voltage_grids():
    a = models.config1_cell(n_cable=10)
    c = models.config1_cell(n_cable=10)
    (mA, mB), (hA, hB) = models.hh_na_tables(vdivs=1000)
    nA, nB = models.hh_k_tables(vdivs=1000)
    c.gates = [(models.VMIN, models.VMAX, mA, mB), (models.VMIN, models.VMAX, hA, hB),
               (models.VMIN, models.VMAX, nA, nB)]
    with pytest.raises(Exception, match="different grids"):
        Batch([a, c], 25e-6, HS_PREC_MIXED)
