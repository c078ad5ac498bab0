"""hs_process_group: separate drop-in HSolves stepped in one launch; and
the cluster form of the drop-in step (hs_set_cluster_ctas).

MOOSE's Clock calls the process of every HSolve on a tick in turn
(scheduling/Clock.cpp:872-921); the group call steps them together, one
CTA (or cluster) per solver, each exactly as hs_process steps it alone.
Events pushed and fields written between calls, recording and spikes are
each solver's own, so a group is bit-identical to the same solvers stepped
one by one.  A cell stepped by a thread-block cluster (its channel and row
work shared by the CTAs, the elimination on one) is bit-identical to the
one-CTA step, and so to the oracle where no libm call is on the path;
from 4,096 compartments on, the cluster also shares the elimination's wide
waves and levels (5,000- and 4,500-compartment cells below, and the
20,000-compartment edge case).
"""
import numpy as np
import pytest

from moose_gb300 import _native, models
from moose_gb300.hsolve import HSolve, process_group
from oracle import OracleCell

pytestmark = pytest.mark.gpu

DT = 25e-6


def _models():
    kca = models.kca_2d_tables(vdivs=300, cadivs=300)
    out = []
    for i, n in enumerate((1, 40, 300, 900, 2500, 64, 5, 1200)):
        rng = np.random.default_rng([13, i])
        if n < 50:
            parent, d, L = models.cable_morphology(n)
        else:
            parent, d, L = models.branched_morphology(rng, n, 0.5, 4)
        out.append(models.active_cell(parent, d, L, inject=float(rng.uniform(0.2e-9, 1.0e-9)), n_syn=12,
                                      rng=rng, t_end=0.05, kca_tables=kca, syn_rate=30.0))
    return out


def _drive(ms, grouped, ctas=0):
    hs = []
    for m in ms:
        h = HSolve(m, dt=DT)
        h.target = m.seed
        h.cluster_ctas = ctas
        h.record([0, m.n_compt - 1], 10, 61)
        h.reinit(DT)
        hs.append(h)
    rng = np.random.default_rng(3)
    for step in range(0, 600, 100):
        for k, (h, m) in enumerate(zip(hs, ms)):
            if (k + step // 100) % 3 == 0:
                h.push_events([k % 12, (k + 5) % 12], [DT * (step + 20 + k), DT * (step + 35)], [2e-9, 1e-9])
            if (k + step // 100) % 4 == 1:
                h.compartment(m.n_compt // 2).inject = float(rng.uniform(0.0, 2e-9))
        if grouped:
            process_group(hs, 100)
        else:
            for h in hs:
                h.process(100)
    out = []
    for h in hs:
        h.sync()
        out.append((h.vm(), h.ca(), h.trace(), h.spikes()))
        h.close()
    return out


def test_group_bit_identical_to_each_solver_alone():
    ms = _models()
    alone = _drive(ms, False)
    group = _drive(ms, True)
    fired = 0
    for a, g in zip(alone, group):
        assert np.array_equal(a[0], g[0])
        assert np.array_equal(a[1], g[1])
        assert np.array_equal(a[2], g[2])
        for x, y in zip(a[3], g[3]):
            assert np.array_equal(x, y)
        fired += len(a[3][0])
    assert fired > 0


def test_group_interleaves_with_single_calls():
    """A group call orders itself after the work queued on every member's
    stream and before what is queued after it."""
    ms = _models()[:4]
    hs = []
    for m in ms:
        h = HSolve(m, dt=DT)
        h.target = m.seed
        h.reinit(DT)
        hs.append(h)
    hs[2].process(50)
    for h in (hs[0], hs[1], hs[3]):
        h.process(50)
    process_group([hs[3], hs[1], hs[0], hs[2]], 250)
    process_group(hs[:2], 300)
    for h in hs[2:]:
        h.process(300)
    for h in hs:
        h.sync()
        # no events or writes here: compare against a plain 600-step run
        h2 = HSolve(h.model, dt=DT)
        h2.target = h.model.seed
        h2.reinit(DT)
        h2.process(600)
        h2.sync()
        assert np.array_equal(h.vm(), h2.vm())
        h2.close()
        h.close()


def test_group_checks_its_members():
    ms = _models()[:2]
    hs = [HSolve(m, dt=DT) for m in ms]
    for h, m in zip(hs, ms):
        h.target = m.seed
    hs[0].reinit(DT)
    with pytest.raises(_native.HsError):
        process_group(hs, 10)                  # hs[1] not reinited
    hs[1].reinit(DT)
    with pytest.raises(_native.HsError):
        process_group([hs[0], hs[1], hs[0]], 10)
    process_group([], 10)
    process_group(hs, 0)
    for h in hs:
        h.close()


def test_cluster_sizes_by_rule():
    ms = _models()
    got = []
    for m in ms:
        h = HSolve(m, dt=DT)
        h.target = m.seed
        got.append(h.cluster_ctas)
        h.cluster_ctas = 3
        assert h.cluster_ctas == 3
        with pytest.raises(_native.HsError):
            h.cluster_ctas = 9
        h.close()
    assert got == [1 if m.n_compt < 1024 else min(8, m.n_compt // 512) for m in ms]
    assert max(got) > 1


@pytest.mark.parametrize("ctas", [2, 3, 5, 8])
def test_cluster_step_bit_identical_to_one_cta(ctas):
    rng = np.random.default_rng([17, ctas])
    parent, d, L = models.branched_morphology(rng, 5000, 0.5, 4)     # wide waves shared by the cluster
    m = models.active_cell(parent, d, L, inject=0.6e-9, n_syn=40, rng=rng, t_end=0.05,
                           kca_tables=models.kca_2d_tables(vdivs=300, cadivs=300), syn_rate=30.0)
    one = _drive([m], False, ctas=1)[0]
    many = _drive([m], False, ctas=ctas)[0]
    for a, b in zip(one[:3], many[:3]):
        assert np.array_equal(a, b)
    for x, y in zip(one[3], many[3]):
        assert np.array_equal(x, y)


def test_cluster_step_bit_exact_with_oracle():
    """No HHChannel2D (its exp is libm's on the host): the cluster step
    equals the oracle bit for bit, Vm and Ca, every 100 steps."""
    rng = np.random.default_rng(29)
    parent, d, L = models.branched_morphology(rng, 4500, 0.5, 4)
    m = models.active_cell(parent, d, L, inject=1.0e-9, gca=10.0, gkca=0.0, n_syn=20, rng=rng,
                           t_end=0.05, syn_rate=40.0)
    for k in list(vars(m)):
        if k.startswith("c2d_"):
            setattr(m, k, getattr(m, k)[:0])
    m.gates2d = []
    h = HSolve(m, dt=DT)
    h.target = m.seed
    h.cluster_ctas = 8
    h.reinit(DT)
    oc = OracleCell(m, DT)
    oc.reinit(DT)
    for _ in range(6):
        h.process(100)
        oc.step(100)
        assert np.array_equal(h.vm(), oc.vm())
        assert np.array_equal(h.ca(), oc.ca())
    h.close()


def _clock(ms, use_group, pattern):
    """A clock loop of one-step calls: each step either the whole tick as
    one group or every solver's own process, with field reads and writes
    between steps; `pattern` also alternates two overlapping groups whose
    first members differ (launches on different streams)."""
    hs = []
    for m in ms:
        h = HSolve(m, dt=DT)
        h.target = m.seed
        h.reinit(DT)
        hs.append(h)
    seen = []
    for step in range(60):
        if use_group:
            if pattern and step % 2:
                process_group([hs[2], hs[0]], 1)
                process_group([hs[1], hs[3]], 1)
            else:
                process_group(hs, 1)
        else:
            for h in hs:
                h.process(1)
        if step % 7 == 3:
            hs[1].compartment(0).inject = 1e-9 * (step % 3)
            seen.append(hs[0].compartment(hs[0].model.n_compt - 1).Vm)
        if step % 11 == 5:
            seen.append(float(hs[2].vm().sum()))
    out = [h.vm() for h in hs]
    for h in hs:
        h.close()
    return out, seen


@pytest.mark.parametrize("pattern", [False, True])
def test_one_step_group_calls_with_field_access_between(pattern):
    ms = _models()[2:6]
    a, sa = _clock(ms, False, pattern)
    b, sb = _clock(ms, True, pattern)
    assert sa == sb
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
