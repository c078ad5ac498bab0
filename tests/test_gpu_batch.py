"""Batched HSolve on the GPU.

FP64 batch: every cell bit-identical to its own drop-in HSolve (same
arithmetic, one warp per cell instead of one CTA).
Mixed batch: |dVm| <= 0.1 mV against the FP64 oracle over the whole run and
spike times within 0.05 ms, the tolerances of the mixed-precision workload.
"""
import numpy as np
import pytest

from moose_gb300 import models
from moose_gb300.abi import (FIELDS, HS_KIND_CHAN, HS_KIND_CHAN2D, HS_KIND_SYNCHAN, HS_PREC_FP64,
                              HS_PREC_MIXED)
from moose_gb300.batch import Batch
from moose_gb300.hsolve import HSolve
from oracle import OracleCell

pytestmark = pytest.mark.gpu

DT = 25e-6


def small_population(n_cells, seed, n_syn=0, t_end=0.05, max_children=4, lo=20, hi=300):
    rng = np.random.default_rng(seed)
    kA, kB = models.kca_2d_tables(vdivs=300, cadivs=300)
    cells = []
    for i in range(n_cells):
        crng = np.random.default_rng([seed, i])
        n = int(crng.integers(lo, hi))
        parent, d, L = models.branched_morphology(crng, n, 0.5, max_children)
        cells.append(models.active_cell(parent, d, L, inject=float(crng.uniform(0.2e-9, 1e-9)),
                                        n_syn=n_syn, rng=crng, t_end=t_end, kca_tables=(kA, kB),
                                        syn_rate=40.0))
    return cells


def test_fp64_batch_matches_dropin_bit_exact():
    cells = small_population(12, 3, n_syn=6)
    b = Batch(cells, DT, HS_PREC_FP64, threads_per_cta=64, ctas_per_sm=1, steps_per_launch=37)
    b.reinit(DT)
    b.process(400)
    for i, m in enumerate(cells):
        h = HSolve(m, dt=DT)
        h.target = m.seed
        h.reinit(DT)
        h.process(400)
        assert np.array_equal(b.vm(i), h.vm()), "cell %d" % i
        assert np.array_equal(b.ca(i), h.ca()), "cell %d" % i


def test_fp64_batch_graph_and_chunks_agree():
    cells = small_population(5, 4)
    a = Batch(cells, DT, HS_PREC_FP64, steps_per_launch=50, use_graph=True)
    c = Batch(cells, DT, HS_PREC_FP64, steps_per_launch=7, use_graph=False)
    a.reinit(DT)
    c.reinit(DT)
    a.process(300)
    for _ in range(6):
        c.process(50)
    for i in range(len(cells)):
        assert np.array_equal(a.vm(i), c.vm(i))


def test_mixed_batch_within_tolerance_of_fp64_oracle():
    cells = small_population(16, 5, n_syn=8, t_end=0.1)
    b = Batch(cells, DT, HS_PREC_MIXED, steps_per_launch=100)
    b.reinit(DT)
    nsteps, chunk = 4000, 100
    oracles = []
    for m in cells:
        oc = OracleCell(m, DT)
        oc.reinit(DT)
        oracles.append(oc)
    worst = 0.0
    for _ in range(nsteps // chunk):
        b.process(chunk)
        for i, oc in enumerate(oracles):
            oc.step(chunk)
            worst = max(worst, float(np.abs(b.vm(i) - oc.vm()).max()))
    assert worst <= 1e-4, "max |dVm| = %g V" % worst
    cell_ids, gens, t = b.spikes()
    for i, oc in enumerate(oracles):
        ref = oc.spikes()[1]
        got = np.sort(t[cell_ids == i])
        assert len(got) == len(ref), "cell %d spike count %d vs %d" % (i, len(got), len(ref))
        if len(ref):
            assert np.abs(got - ref).max() <= 5e-5


def test_mixed_recording_and_tuning():
    cells = small_population(6, 6)
    b = Batch(cells, DT, HS_PREC_MIXED)
    b.record([0, 0, 3, 5], [0, 4, 0, 2], 10, 51)
    b.reinit(DT)
    b.process(200)
    # a new launch shape without a new packing keeps the state
    b.tune(threads_per_cta=128, steps_per_launch=25)
    b.process(300)
    tr, cols = b.trace()
    assert tr.shape == (51, 4)
    assert cols == [(0, 0), (0, 4), (3, 0), (5, 2)]
    assert np.array_equal(tr[-1], [b.vm(c)[m] for c, m in cols])
    ms, n = b.kernel_time()
    assert n >= 1 and ms > 0


def test_mixed_results_do_not_depend_on_packing():
    """A cell's result is the same alone, in a large mix, in small shared
    forests, in global forests and under any launch shape (bit-identical:
    every node's arithmetic is fixed by its own cell)."""
    cells = small_population(12, 7, n_syn=4)
    a = Batch(cells, DT, HS_PREC_MIXED)
    c = Batch(cells, DT, HS_PREC_MIXED, threads_per_cta=256, ctas_per_sm=2, forest_nodes=64)
    alone = Batch([cells[3]], DT, HS_PREC_MIXED, threads_per_cta=96)
    for x in (a, c, alone):
        x.reinit(DT)
        x.process(500)
    for i in range(len(cells)):
        assert np.array_equal(a.vm(i), c.vm(i)), i
    assert np.array_equal(alone.vm(0), a.vm(3))
    # repacking an existing batch starts it over
    a.tune(ctas_per_sm=2, forest_nodes=128)
    with pytest.raises(Exception):
        a.process(10)
    a.reinit(DT)
    a.process(500)
    for i in range(len(cells)):
        assert np.array_equal(a.vm(i), c.vm(i)), i


def test_mixed_edge_cases_against_the_oracle():
    """One- and two-compartment cells, and an unbranched 1,500-compartment
    cable (more tree levels than the kernel keeps in shared memory), in one
    mixed batch: within the mixed-precision tolerance of the FP64 oracle."""
    kA, kB = models.kca_2d_tables(vdivs=300, cadivs=300)
    cells = []
    for n in (1, 2):
        parent = np.arange(-1, n - 1, dtype=np.int32)
        d = np.full(n, 2e-6)
        L = np.full(n, 10e-6)
        cells.append(models.active_cell(parent, d, L, inject=0.05e-9, kca_tables=(kA, kB), t_end=0.05))
    parent, d, L = models.cable_morphology(1499)
    cells.append(models.active_cell(parent, d, L, inject=0.8e-9, kca_tables=(kA, kB), t_end=0.05))
    b = Batch(cells, DT, HS_PREC_MIXED, steps_per_launch=50)
    b.reinit(DT)
    oracles = []
    for m in cells:
        oc = OracleCell(m, DT)
        oc.reinit(DT)
        oracles.append(oc)
    worst = 0.0
    for _ in range(8):
        b.process(250)
        for i, oc in enumerate(oracles):
            oc.step(250)
            worst = max(worst, float(np.abs(b.vm(i) - oc.vm()).max()))
    assert worst <= 1e-4, "max |dVm| = %g V" % worst


def test_concurrent_batches_keep_their_own_prototypes():
    """Two mixed batches with different channel sets on one GPU: creating
    and stepping the second does not change what the first computes (each
    batch carries its own channel, K(Ca) and SynChan tables)."""
    cells_a = small_population(5, 31, n_syn=4)
    cells_b = [models.config1_cell(n_cable=40, inject=0.4e-9) for _ in range(3)]
    ref = Batch(cells_a, DT, HS_PREC_MIXED)
    ref.reinit(DT)
    ref.process(400)
    a = Batch(cells_a, DT, HS_PREC_MIXED)
    a.reinit(DT)
    a.process(200)
    b = Batch(cells_b, DT, HS_PREC_MIXED)
    b.reinit(DT)
    b.process(100)
    a.process(200)
    b.process(100)
    for i in range(len(cells_a)):
        assert np.array_equal(a.vm(i), ref.vm(i)), i
    solo = Batch(cells_b, DT, HS_PREC_MIXED)
    solo.reinit(DT)
    solo.process(200)
    for i in range(len(cells_b)):
        assert np.array_equal(b.vm(i), solo.vm(i)), i


def test_modulation_writes():
    """hs_batch_set_modulation (an Adaptor driving channel modulation) on
    HHChannels (one write of 0, which setHHmodulation ignores), HHChannel2Ds
    and SynChans part way through a run: the FP64 batch bit-exact with the
    drop-in given the same field writes, the mixed batch within 0.1 mV of
    the oracle given them."""
    cells = small_population(6, 9, n_syn=6, t_end=0.1)
    writes = []
    for c, m in enumerate(cells):
        writes += [(HS_KIND_CHAN, c, 0, 1.3), (HS_KIND_CHAN, c, 4, 0.0), (HS_KIND_CHAN, c, 7, 0.6),
                   (HS_KIND_CHAN2D, c, 2, 0.5), (HS_KIND_SYNCHAN, c, 1, 2.0)]
    fmod = FIELDS["modulation"]

    def apply_batch(b):
        for kind in (HS_KIND_CHAN, HS_KIND_CHAN2D, HS_KIND_SYNCHAN):
            w = [x for x in writes if x[0] == kind]
            b.set_modulation(kind, [x[1] for x in w], [x[2] for x in w], [x[3] for x in w])

    fb = Batch(cells, DT, HS_PREC_FP64)
    mb = Batch(cells, DT, HS_PREC_MIXED)
    for b in (fb, mb):
        b.reinit(DT)
        b.process(300)
        apply_batch(b)
        b.process(700)
    for c, m in enumerate(cells):
        h = HSolve(m, dt=DT)
        h.target = m.seed
        h.reinit(DT)
        h.process(300)
        oc = OracleCell(m, DT)
        oc.reinit(DT)
        oc.step(300)
        for kind, cc, i, v in writes:
            if cc == c:
                h._set(kind, fmod, i, v)
                oc.set(kind, fmod, i, v)
        h.process(700)
        oc.step(700)
        assert np.array_equal(fb.vm(c), h.vm()), c
        assert np.abs(mb.vm(c) - oc.vm()).max() <= 1e-4, c


@pytest.mark.parametrize("prec", [HS_PREC_FP64, HS_PREC_MIXED])
def test_failed_record_keeps_previous_recording(prec):
    """A rejected hs_batch_record leaves the previous recording in place and
    the batch keeps stepping into live buffers."""
    from moose_gb300._native import HsError
    cells = small_population(4, 8)
    b = Batch(cells, DT, prec)
    b.record([0, 2], [0, 3], 10, 31)
    b.reinit(DT)
    b.process(100)
    with pytest.raises(HsError):
        b.record([0, 9], [0, 0], 10, 31)
    with pytest.raises(HsError):
        b.record([0, 1], [0, 100_000], 10, 31)
    b.process(200)
    tr, cols = b.trace()
    assert tr.shape == (31, 2)
    assert np.array_equal(tr[-1], [b.vm(c)[m] for c, m in cols])
    b.close()


def test_bounded_wait_gives_up_with_etimeout():
    """The split step's eliminator waits are bounded: with a limit of one
    sleep round (~128 ns, shorter than the assembly of any level) every
    eliminator gives up at its first wait, the launch still ends, and
    hs_batch_sync reports HS_ETIMEOUT; nothing faults.  reinit clears the
    flag, and a fresh batch of the same cells steps correctly afterwards."""
    from moose_gb300._native import HsError
    from moose_gb300.abi import HS_ETIMEOUT
    cells = small_population(6, 12, lo=100, hi=300)
    b = Batch(cells, DT, HS_PREC_MIXED, wait_rounds=1, steps_per_launch=20)
    b.reinit(DT)
    b.process(100)
    with pytest.raises(HsError) as ei:
        b.sync()
    assert ei.value.code == HS_ETIMEOUT
    b.reinit(DT)
    b.sync()                       # the flag is cleared by reinit
    b.close()
    good = Batch(cells, DT, HS_PREC_MIXED, steps_per_launch=20)
    good.reinit(DT)
    good.process(200)
    good.sync()
    for i, m in enumerate(cells):
        o = OracleCell(m, DT)
        o.reinit(DT)
        o.step(200)
        assert np.abs(good.vm(i) - o.vm()).max() <= 1e-4
    good.close()


def test_fp64_batch_whole_cta_and_warp_cells_bit_exact():
    """The FP64 batch steps its largest cells with a whole CTA each and the
    rest one warp per cell (the packing chooses by cost): a mix of two
    3,000-compartment cells and small ones is bit-identical to per-cell
    drop-ins whichever form stepped each cell."""
    small = small_population(10, 21, n_syn=4, lo=20, hi=200)
    big = small_population(2, 22, n_syn=4, lo=3000, hi=3001)
    cells = big[:1] + small + big[1:]
    b = Batch(cells, DT, HS_PREC_FP64, steps_per_launch=60)
    b.reinit(DT)
    b.process(300)
    for i, m in enumerate(cells):
        h = HSolve(m, dt=DT)
        h.target = m.seed
        h.reinit(DT)
        h.process(300)
        assert np.array_equal(b.vm(i), h.vm()), "cell %d" % i
        assert np.array_equal(b.ca(i), h.ca()), "cell %d" % i
        h.close()
    b.close()
