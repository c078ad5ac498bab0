"""Edge cases of size and shape on the GPU, against the oracle.

* A junction of rank 41 (a soma with 40 three-compartment dendrites): the
  reference's generic rank >= 3 operand path at its widest.
* A 20,000-compartment branched cell: larger than any workload cell, and
  larger than a mixed-batch forest in shared memory.
* 400 SynChans on one compartment, with events tied in time.
* The mixed batch's forest limit: a cell of more than 65,535 star-form
  nodes is refused at creation (HS_ENOTSUP), nothing is launched.

Bars as elsewhere: the FP64 drop-in bit for bit with the oracle where no
libm call is on the path, the FP64 batch bit-identical to the drop-in, the
mixed batch within 0.1 mV of the oracle.
"""
import numpy as np
import pytest

from moose_gb300 import _native, models
from moose_gb300.abi import HS_PREC_FP64, HS_PREC_MIXED
from moose_gb300.batch import Batch
from moose_gb300.hsolve import HSolve
from oracle import OracleCell

pytestmark = pytest.mark.gpu

DT = 25e-6


def _libm_free(m):
    """Drop the K(Ca) 2-D channel (its exp differs between device and host
    libm by an ulp) so that the whole path is bit-comparable."""
    for k in list(vars(m)):
        if k.startswith("c2d_"):
            setattr(m, k, getattr(m, k)[:0])
    m.gates2d = []
    return m


def _star_cell(n_dend=40, seg=3):
    parent = [-1]
    for _ in range(n_dend):
        p = 0
        for _ in range(seg):
            parent.append(p)
            p = len(parent) - 1
    parent = np.array(parent, np.int32)
    n = len(parent)
    d = np.full(n, 1.5e-6)
    L = np.full(n, 12e-6)
    d[0], L[0] = 20e-6, 20e-6
    return _libm_free(models.active_cell(parent, d, L, inject=0.8e-9, gca=10.0, gkca=0.0, t_end=0.05))


def _run_pair(m, nsteps, chunk):
    h = HSolve(m, dt=DT)
    h.target = m.seed
    h.reinit(DT)
    oc = OracleCell(m, DT)
    oc.reinit(DT)
    for _ in range(nsteps // chunk):
        h.process(chunk)
        oc.step(chunk)
        assert np.array_equal(h.vm(), oc.vm())
    return h, oc


def test_rank_41_junction_dropin_batch_and_mixed():
    m = _star_cell()
    assert np.bincount(m.parent[m.parent >= 0]).max() == 40
    h, oc = _run_pair(m, 800, 200)
    assert np.array_equal(h.ca(), oc.ca())
    b = Batch([m], DT, HS_PREC_FP64)
    b.reinit(DT)
    b.process(800)
    assert np.array_equal(b.vm(0), h.vm())
    mx = Batch([m], DT, HS_PREC_MIXED)
    mx.reinit(DT)
    mx.process(800)
    assert float(np.abs(mx.vm(0) - oc.vm()).max()) <= 1e-4
    for x in (h, b, mx):
        x.close()


def test_20000_compartment_cell():
    rng = np.random.default_rng(77)
    parent, d, L = models.branched_morphology(rng, 20000, 0.5, 3)
    m = _libm_free(models.active_cell(parent, d, L, inject=1.0e-9, gca=10.0, gkca=0.0, t_end=0.05))
    h, oc = _run_pair(m, 200, 100)
    b = Batch([m], DT, HS_PREC_FP64)
    b.reinit(DT)
    b.process(200)
    assert np.array_equal(b.vm(0), h.vm())
    mx = Batch([m], DT, HS_PREC_MIXED)
    mx.reinit(DT)
    oc = OracleCell(m, DT)
    oc.reinit(DT)
    worst = 0.0
    for _ in range(4):
        mx.process(500)
        oc.step(500)
        worst = max(worst, float(np.abs(mx.vm(0) - oc.vm()).max()))
    assert worst <= 1e-4, worst
    for x in (h, b, mx):
        x.close()


def test_400_synchans_on_one_compartment_with_tied_events():
    parent, d, L = models.cable_morphology(20)
    m = _libm_free(models.active_cell(parent, d, L, inject=0.0, n_syn=400, syn_rate=20.0, t_end=0.05,
                                      rng=np.random.default_rng(5), gca=10.0, gkca=0.0))
    m.syn_compt[:] = 3
    # every event at one of a few times: many ties on each SynChan
    m.ev_time = np.round(m.ev_time / 2e-3) * 2e-3
    h, oc = _run_pair(m, 2000, 500)
    b = Batch([m, m], DT, HS_PREC_FP64)
    b.reinit(DT)
    b.process(2000)
    assert np.array_equal(b.vm(0), h.vm()) and np.array_equal(b.vm(1), h.vm())
    for x in (h, b):
        x.close()


def test_mixed_batch_refuses_a_cell_beyond_the_forest_limit():
    parent, d, L = models.cable_morphology(70000)
    m = models.active_cell(parent, d, L, inject=0.5e-9, t_end=0.01)
    with pytest.raises(_native.HsError):
        Batch([m], DT, HS_PREC_MIXED)
