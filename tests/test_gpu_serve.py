"""Serving loop on the GPU: each request's result is the same alone and in
the mix (tolerance: bit-identical, since a cell's arithmetic depends only on
the cell), per-cell stop steps freeze a cell exactly, and the memory estimate
used for admission bounds what a cohort allocates."""
import numpy as np
import pytest

from moose_gb300 import models
from moose_gb300.abi import HS_PREC_MIXED
from moose_gb300.batch import Batch
from moose_gb300 import serve

pytestmark = pytest.mark.gpu

# cohorts of the serving loop overlap on the GPU only with enough hardware
# work queues; pytest imports every test module before the first test starts
# CUDA, so this takes effect for the whole run
serve.configure_work_queues(32)

DT = 25e-6


def requests(n, seed=11):
    kA, kB = models.kca_2d_tables(vdivs=300, cadivs=300)
    out = []
    for i in range(n):
        rng = np.random.default_rng([seed, i])
        size = int(rng.integers(30, 400))
        steps = int(rng.integers(200, 1600))
        parent, d, L = models.branched_morphology(rng, size, 0.5, 4)
        if i % 2:
            cell = models.active_cell(parent, d, L, inject=float(rng.uniform(0.3e-9, 1e-9)), rng=rng,
                                      t_end=steps * DT, kca_tables=(kA, kB))
        else:
            cell = models.active_cell(parent, d, L, inject=0.0, n_syn=int(rng.integers(50, 200)), rng=rng,
                                      t_end=steps * DT, kca_tables=(kA, kB), syn_rate=60.0)
        out.append(serve.Request(i, cell, steps, arrival=float(2 * i)))
    return out


def tick_server(**kw):
    """A server whose clock is its tick count (arrival times are in ticks)."""
    box = []
    srv = serve.Server(DT, clock=lambda: float(box[0].ticks) if box else 0.0, **kw)
    box.append(srv)
    return srv


def test_each_request_same_alone_and_in_the_mix():
    reqs = requests(8)
    mix = tick_server(chunk=100, record_stride=10).run(reqs)
    assert sorted(r.rid for r in mix) == list(range(8))
    by_id = {r.rid: r for r in mix}
    for q in reqs:
        alone = serve.Server(DT, chunk=100, record_stride=10).run(
            [serve.Request(q.rid, q.cell, q.n_steps)], real_time=False)[0]
        m = by_id[q.rid]
        assert len(m.vm) == q.n_steps // 10 + 1
        assert np.array_equal(m.vm, alone.vm), q.rid
        assert np.array_equal(m.spike_times, alone.spike_times), q.rid
    assert any(len(r.spike_times) for r in mix)


def test_stop_steps_freeze_a_cell_exactly():
    reqs = requests(4, seed=3)
    cells = [r.cell for r in reqs]
    b = Batch(cells, DT, HS_PREC_MIXED, steps_per_launch=64)
    b.set_stop_steps([150, None, 333, 0])
    b.reinit(DT)
    b.process(500)
    steps = b.steps()
    assert list(steps) == [150, 500, 333, 0]
    for i, n in ((0, 150), (2, 333)):
        ref = Batch([cells[i]], DT, HS_PREC_MIXED, steps_per_launch=64)
        ref.reinit(DT)
        ref.process(n)
        assert np.array_equal(b.vm(i), ref.vm(0))
        ref.close()
    init = Batch([cells[3]], DT, HS_PREC_MIXED)
    init.reinit(DT)
    assert np.array_equal(b.vm(3), init.vm(0))


def test_memory_estimate_bounds_the_cohort():
    reqs = requests(6, seed=5)
    over = serve.cohort_overhead(reqs[0].cell)
    for q in reqs[:3]:
        c = serve._Cohort([q], DT, 10, 100, 0.0, {})
        assert c.bytes <= over + serve.estimate_bytes(q.cell, q.n_steps, 10), (c.bytes, q.cell.n_compt)
        c.close()
    c = serve._Cohort(reqs, DT, 10, 100, 0.0, {})
    assert c.bytes <= over + sum(serve.estimate_bytes(q.cell, q.n_steps, 10) for q in reqs)
    c.close()
