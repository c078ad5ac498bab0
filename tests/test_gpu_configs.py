"""Parity at the workloads' own sizes, on the GPU, against the oracle (the
CPU restatement of the reference HSolve, pinned bit-exact to the reference
build) and against the FP64 drop-in.

* 256-cell workload (binary branching, 100..1,000 compartments, HH + Ca(HVA)
  + K(Ca) HHChannel2D + CaConc, 0.1..1 nA soma step): 16 whole cells, each
  its own FP64 drop-in HSolve, for the full 1 s (40,000 steps) against the
  oracle: Vm within 1e-9 relative (device exp vs glibc exp in the K(Ca)
  gate), identical spike counts.
* 4,096-cell workload (log-uniform 50..5,000 compartments, junctions of up
  to 4 children): the FP64 batch bit-identical to per-cell drop-ins on 8
  cells of 1,000..5,000 compartments with rank-3 and rank-4 junctions.
* mixed precision at the synaptic workload's resolution (3000-division V
  and Ca tables, 200 SynChans at 5 Hz per cell, dt 25 us, 0.25 s): a
  5,000-compartment unbranched cable and two of the workload's cells
  against the oracle: max |dVm| <= 0.1 mV over every step at the soma and
  over every compartment every 500 steps, spike times within 0.05 ms,
  identical spike counts.
"""
import numpy as np
import pytest

import oracle_pool
from moose_gb300 import models
from moose_gb300.abi import HS_PREC_FP64, HS_PREC_MIXED
from moose_gb300.batch import Batch
from moose_gb300.hsolve import HSolve

pytestmark = pytest.mark.gpu

DT = 25e-6
SEED = 1


def _rel_close(got, ref, rtol=1e-9):
    return np.all(np.abs(got - ref) <= rtol * np.maximum(np.abs(ref), 1e-3))


def test_config2_dropins_full_second_vs_oracle():
    nsteps, stride = 40000, 100
    ids = list(range(0, 256, 16))
    jobs = [("workload", (2, SEED, i, 1.0, 256), nsteps, stride, 0) for i in ids]
    ref = oracle_pool.run(jobs)
    sizes, _, _ = models.population_sizes(2, SEED, 256)
    hs = []
    for i in ids:
        m = models.make_cell(2, SEED, i, n_cells=256, t_end=1.0, sizes=sizes)
        h = HSolve(m, dt=DT)
        h.target = m.seed
        h.record([0], stride, nsteps // stride + 1)
        h.reinit(DT)
        hs.append((m, h))
    for _, h in hs:
        h.process(nsteps)          # every instance on its own stream, concurrently
    spikes_total = 0
    for (m, h), r in zip(hs, ref):
        h.sync()
        tr = h.trace()[0]
        assert tr.shape == r["soma"].shape
        assert _rel_close(tr, r["soma"]), np.abs(tr - r["soma"]).max()
        assert _rel_close(h.vm(), r["vm"])
        assert _rel_close(h.ca(), r["ca"], 1e-9)
        _, t = h.spikes()
        assert len(t) == len(r["spikes"])
        spikes_total += len(t)
        h.close()
    assert spikes_total > 0


def _children_counts(parent):
    return np.bincount(parent[parent >= 0], minlength=len(parent))


def test_config3_fp64_batch_bit_identical_on_large_cells():
    sizes, _, _ = models.population_sizes(3, SEED, 4096)
    ids = [i for i in range(4096) if 1000 <= sizes[i] <= 5000][:8]
    assert len(ids) == 8
    cells = [models.make_cell(3, SEED, i, n_cells=4096, t_end=0.1, sizes=sizes) for i in ids]
    kids = [_children_counts(m.parent) for m in cells]
    assert max(int(k.max()) for k in kids) == 4            # rank-4 junctions
    assert sum(int((k == 3).sum()) for k in kids) > 0       # rank-3 junctions
    b = Batch(cells, DT, HS_PREC_FP64)
    b.reinit(DT)
    hs = []
    for m in cells:
        h = HSolve(m, dt=DT)
        h.target = m.seed
        h.reinit(DT)
        hs.append(h)
    nsteps = 2000
    b.process(nsteps)
    for h in hs:
        h.process(nsteps)
    b.sync()
    vall = b.read_all("Vm")
    off = 0
    for k, (m, h) in enumerate(zip(cells, hs)):
        h.sync()
        assert np.array_equal(b.vm(k), h.vm()), k
        assert np.array_equal(vall[off:off + m.n_compt], h.vm()), k
        assert np.array_equal(b.ca(k), h.ca()), k
        off += m.n_compt
        h.close()
    b.close()


def test_mixed_at_synaptic_workload_resolution_vs_oracle():
    nsteps, full_every = 10000, 500
    t_end = nsteps * DT + 0.01
    sizes, _, _ = models.population_sizes(4, SEED, 4096)
    small = next(i for i in range(4096) if 150 <= sizes[i] <= 300)
    large = next(i for i in range(4096) if sizes[i] >= 4000)
    jobs = [("cable", (5000, SEED, t_end), nsteps, 1, full_every),
            ("workload", (4, SEED, small, t_end, 4096), nsteps, 1, full_every),
            ("workload", (4, SEED, large, t_end, 4096), nsteps, 1, full_every)]
    ref = oracle_pool.run(jobs)
    cells = [oracle_pool.cable_cell(5000, SEED, t_end),
             models.make_cell(4, SEED, small, n_cells=4096, t_end=t_end, sizes=sizes),
             models.make_cell(4, SEED, large, n_cells=4096, t_end=t_end, sizes=sizes)]
    assert [len(m.syn_compt) for m in cells] == [200, 200, 200]
    assert all(len(g[2]) == 3001 for m in cells for g in m.gates)
    assert all(np.shape(g[4]) == (3001, 3001) for m in cells for g in m.gates2d)
    b = Batch(cells, DT, HS_PREC_MIXED)
    b.record(np.arange(3), np.zeros(3, np.uint32), 1, nsteps + 1)
    b.reinit(DT)
    worst_full = 0.0
    for k in range(nsteps // full_every):
        b.process(full_every)
        for c, r in enumerate(ref):
            worst_full = max(worst_full, float(np.abs(b.vm(c) - r["full"][k]).max()))
    tr, cols = b.trace()
    assert [c for c, _ in cols] == [0, 1, 2]
    worst_soma = max(float(np.abs(tr[:, c] - ref[c]["soma"]).max()) for c in range(3))
    cell, _, t = b.spikes()
    shift, n_spikes = 0.0, 0
    for c in range(3):
        mine = np.sort(t[cell == c])
        assert len(mine) == len(ref[c]["spikes"]), (c, len(mine), len(ref[c]["spikes"]))
        if len(mine):
            shift = max(shift, float(np.abs(mine - ref[c]["spikes"]).max()))
        n_spikes += len(mine)
    b.close()
    assert n_spikes > 0
    assert worst_soma <= 1e-4, worst_soma
    assert worst_full <= 1e-4, worst_full
    assert shift <= 5e-5, shift
