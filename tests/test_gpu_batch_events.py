"""Synaptic events pushed at run time into batches (hs_batch_push_events,
SimpleSynHandler::addSpike for many cells at once).

FP64 batch: every cell bit-identical to its own drop-in HSolve receiving the
same pushes through hs_push_events (itself bit-exact with the oracle and the
reference's active_events golden), across growing pushes, ties, events at
+-inf, events already in the past, and a reinit that drops the queue.
Mixed batch: within 0.1 mV and 0.05 ms of the FP64 oracle receiving the
same pushes, identical spike counts.
"""
import numpy as np
import pytest

from moose_gb300 import _native
from moose_gb300.abi import HS_PREC_FP64, HS_PREC_MIXED
from moose_gb300.batch import Batch
from moose_gb300.hsolve import HSolve
from oracle import OracleCell
from test_gpu_batch import small_population

pytestmark = pytest.mark.gpu

DT = 25e-6


def _pushes(rng, cells, step, n):
    """n events on random SynChans of random cells around the current time,
    an eighth of them tied on one SynChan with different weights."""
    cell = rng.integers(0, len(cells), n)
    syn = np.array([rng.integers(0, len(cells[c].syn_compt)) for c in cell])
    t = DT * step + rng.uniform(-2e-3, 6e-3, n)
    w = rng.uniform(0.5e-9, 3e-9, n)
    q = max(1, n // 8)
    cell[:q] = cell[0]
    syn[:q] = syn[0]
    t[:q] = DT * (step + 3) + 0.5 * DT
    return cell, syn, t, w


def _deliver(targets, cell, syn, t, w):
    for c, tgt in enumerate(targets):
        sel = cell == c
        if sel.any():
            tgt.push_events(syn[sel], t[sel], w[sel])


def test_fp64_batch_runtime_events_bit_identical_to_dropins():
    cells = small_population(8, 11, n_syn=6)
    b = Batch(cells, DT, HS_PREC_FP64, steps_per_launch=50)
    hs = []
    for m in cells:
        h = HSolve(m, dt=DT)
        h.target = m.seed
        hs.append(h)
    rng = np.random.default_rng(3)
    for rnd in range(2):
        b.reinit(DT)
        for h in hs:
            h.reinit(DT)
        step = 0
        for chunk in range(8):
            cell, syn, t, w = _pushes(rng, cells, step, 10 * 3 ** min(chunk, 4))
            if chunk == 2:
                cell = np.concatenate([cell, [1, 2]])
                syn = np.concatenate([syn, [0, 1]])
                t = np.concatenate([t, [-np.inf, np.inf]])
                w = np.concatenate([w, [2e-9, 2e-9]])
            b.push_events(cell, syn, t, w)
            _deliver(hs, cell, syn, t, w)
            b.process(100)
            for h in hs:
                h.process(100)
            step += 100
            for i, h in enumerate(hs):
                assert np.array_equal(b.vm(i), h.vm()), (rnd, chunk, i)
        for i, h in enumerate(hs):
            assert np.array_equal(b.ca(i), h.ca()), i
        bc, _, bt = b.spikes()
        for i, h in enumerate(hs):
            assert np.array_equal(np.sort(bt[bc == i]), np.sort(h.spikes()[1])), i
        # queued but never delivered: dropped by the next reinit on both sides
        cell, syn, t, w = _pushes(rng, cells, step, 50)
        b.push_events(cell, syn, t, w)
        _deliver(hs, cell, syn, t, w)
    assert sum(len(h.spikes()[1]) for h in hs) > 0
    for h in hs:
        h.close()
    b.close()


def test_mixed_batch_runtime_events_vs_oracle():
    cells = small_population(8, 12, n_syn=6, t_end=0.06)
    b = Batch(cells, DT, HS_PREC_MIXED, steps_per_launch=50)
    b.reinit(DT)
    quiet = Batch(cells, DT, HS_PREC_MIXED, steps_per_launch=50)
    quiet.reinit(DT)
    ocs = []
    for m in cells:
        oc = OracleCell(m, DT)
        oc.reinit(DT)
        ocs.append(oc)
    rng = np.random.default_rng(4)
    worst, step = 0.0, 0
    for chunk in range(20):
        cell, syn, t, w = _pushes(rng, cells, step, 60)
        b.push_events(cell, syn, t, w)
        _deliver(ocs, cell, syn, t, w)
        b.process(100)
        quiet.process(100)
        for oc in ocs:
            oc.step(100)
        step += 100
        for i, oc in enumerate(ocs):
            worst = max(worst, float(np.abs(b.vm(i) - oc.vm()).max()))
    assert worst <= 1e-4, worst
    moved = max(float(np.abs(b.vm(i) - quiet.vm(i)).max()) for i in range(len(cells)))
    assert moved > 1e-3          # the pushed events did reach the cells
    bc, _, bt = b.spikes()
    n = 0
    for i, oc in enumerate(ocs):
        ref = oc.spikes()[1]
        got = np.sort(bt[bc == i])
        assert len(got) == len(ref), (i, len(got), len(ref))
        if len(ref):
            assert np.abs(got - ref).max() <= 5e-5
        n += len(ref)
    assert n > 0
    # a reinit drops the queue: the next run equals a batch that never had pushes
    b.push_events([0, 1], [0, 0], [DT * (step + 2)] * 2, [5e-9, 5e-9])
    b.reinit(DT)
    quiet.reinit(DT)
    b.process(300)
    quiet.process(300)
    for i in range(len(cells)):
        assert np.array_equal(b.vm(i), quiet.vm(i)), i
    b.close()
    quiet.close()


@pytest.mark.parametrize("prec", [HS_PREC_FP64, HS_PREC_MIXED])
def test_batch_push_events_rejects_bad_input(prec):
    cells = small_population(3, 13, n_syn=4)
    b = Batch(cells, DT, prec)
    ref = Batch(cells, DT, prec)
    b.reinit(DT)
    ref.reinit(DT)
    with pytest.raises(_native.HsError):
        b.push_events([3], [0], [1e-3], [1e-9])                      # no such cell
    with pytest.raises(_native.HsError):
        b.push_events([0, 1], [0, len(cells[1].syn_compt)], [1e-3, 1e-3], [1e-9, 1e-9])
    with pytest.raises(_native.HsError):
        b.push_events([0, 1], [0, 0], [1e-3, float("nan")], [1e-9, 1e-9])
    with pytest.raises(ValueError):
        b.push_events([0, 1], [0], [1e-3], [1e-9])
    b.push_events([], [], [], [])
    # the rejected calls queued nothing
    b.process(200)
    ref.process(200)
    for i in range(len(cells)):
        assert np.array_equal(b.vm(i), ref.vm(i))
    b.close()
    ref.close()
