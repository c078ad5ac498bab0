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
from moose_gb300 import genesis
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
    this machine's libm) calls libm, else within 1e-9."""
    m = genesis.load_p(path(name), LIB)
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


@pytest.mark.parametrize("group", [("relative_cartesian",) * 3, ("absolute_polar", "spherical_soma")])
def test_mixed_batch_within_tolerance(group):
    """One mixed batch per channel set (a batch shares one rate-table set):
    the full-channel cell at three injects; the two HH-only cells."""
    cells = []
    for k, name in enumerate(group):
        m = genesis.load_p(path(name), LIB)
        m.inject[0] = float(Z["inject"]) * (1.0 + 0.5 * k)
        cells.append(m)
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
