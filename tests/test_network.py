"""moose_gb300.network against three cells the reference coupled by spikes,
each with its own HSolve (tests/golden/make_golden_network.py): stepped in
chunks no longer than the shortest delay, with each chunk's spikes queued
on their targets, the oracle cells reproduce every cell's soma trace and
spike times bit for bit; and the result does not depend on the chunk
length."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from loader import load_model
from moose_gb300.network import Network
from oracle import OracleCell

Z = np.load(os.path.join(GOLDEN, "network_golden.npz"))


class Stepper:
    """An oracle cell with the solver's method names, recording soma Vm."""

    def __init__(self, m, dt):
        self.oc = OracleCell(m, dt)
        self.oc.reinit(dt)
        self.vm = [self.oc.vm()[0]]

    def process(self, n):
        for _ in range(n):
            self.oc.step(1)
            self.vm.append(self.oc.vm()[0])

    def spikes(self):
        return self.oc.spikes()

    def push_events(self, syn, time, weight):
        self.oc.push_events(syn, time, weight)


def _run(chunk=None):
    dt, n = float(Z["dt"]), int(Z["nsteps"])
    cells = [Stepper(load_model(Z, prefix="m%d_" % i), dt) for i in range(3)]
    conns = [(int(a), int(b), int(c), int(d), float(e), float(f)) for a, b, c, d, e, f in Z["connections"]]
    net = Network(cells, conns, dt)
    assert net.chunk == 59                       # 1.5 ms of 25 us steps, strictly inside the delay
    if chunk is not None:
        net.chunk = chunk
    net.run(n)
    return cells


def test_network_reproduces_the_reference_run():
    cells = _run()
    for i, c in enumerate(cells):
        assert np.array_equal(np.array(c.vm), Z["vm%d" % i]), i
        assert np.array_equal(c.spikes()[1], Z["spikes%d" % i]), i
    assert all(len(Z["spikes%d" % i]) > 5 for i in range(3))


@pytest.mark.parametrize("chunk", [1, 17])
def test_chunk_length_does_not_change_the_result(chunk):
    cells = _run(chunk)
    for i, c in enumerate(cells):
        assert np.array_equal(c.spikes()[1], Z["spikes%d" % i]), i


def test_connections_are_checked():
    with pytest.raises(ValueError):
        Network([], [(0, 0, 1, 0, 1e-3, 1.0)], 25e-6)
    with pytest.raises(ValueError):
        Network([object(), object()], [(0, 0, 1, 0, -1e-3, 1.0)], 25e-6)
    assert Network([object()], [(0, 0, 0, 0, 0.0, 1.0)], 25e-6).chunk == 1     # zero delay: one step


class GpuCell:
    """A drop-in HSolve recording its soma Vm every step on the device."""

    def __init__(self, m, dt, n):
        from moose_gb300.hsolve import HSolve
        self.h = HSolve(m, dt=dt)
        self.h.target = m.seed
        self.h.record([0], 1, n + 1)
        self.h.reinit(dt)


@pytest.mark.gpu
def test_network_of_dropin_solvers_on_gpu():
    """The same network with every cell an FP64 drop-in HSolve (the chunks
    through one hs_process_group call each): bit-exact with the reference."""
    dt, n = float(Z["dt"]), int(Z["nsteps"])
    cells = [GpuCell(load_model(Z, prefix="m%d_" % i), dt, n) for i in range(3)]
    conns = [(int(a), int(b), int(c), int(d), float(e), float(f)) for a, b, c, d, e, f in Z["connections"]]
    net = Network([c.h for c in cells], conns, dt)
    assert net._tick is not None
    net.run(n)
    for i, c in enumerate(cells):
        c.h.sync()
        assert np.array_equal(c.h.trace()[0], Z["vm%d" % i]), i
        assert np.array_equal(c.h.spikes()[1], Z["spikes%d" % i]), i
        c.h.close()


class OracleBatch:
    """Oracle cells behind the batch's interface (spikes of all cells in
    one list, events addressed by cell)."""

    def __init__(self, ms, dt):
        self.cells = [Stepper(m, dt) for m in ms]

    def process(self, n):
        for c in self.cells:
            c.process(n)

    def spikes(self):
        cs, gs, ts = [], [], []
        for i, c in enumerate(self.cells):
            g, t = c.spikes()
            cs += [i] * len(t)
            gs += list(g)
            ts += list(t)
        return np.array(cs, np.uint32), np.array(gs, np.uint32), np.array(ts)

    def push_events(self, cells, syn, time, weight):
        for c, k, t, w in zip(cells, syn, time, weight):
            self.cells[int(c)].push_events([k], [t], [w])


def test_batch_network_reproduces_the_reference_run():
    """BatchNetwork over the batch interface: the spikes are read after each
    chunk (the batch lists every cell's spikes, not in time order across
    cells) and pushed in one call."""
    from moose_gb300.network import BatchNetwork
    dt, n = float(Z["dt"]), int(Z["nsteps"])
    b = OracleBatch([load_model(Z, prefix="m%d_" % i) for i in range(3)], dt)
    conns = [(int(a), int(b_), int(c), int(d), float(e), float(f)) for a, b_, c, d, e, f in Z["connections"]]
    net = BatchNetwork(b, conns, dt)
    net.run(n)
    for i, c in enumerate(b.cells):
        assert np.array_equal(np.array(c.vm), Z["vm%d" % i]), i
