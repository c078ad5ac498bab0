"""Cells coupled by spikes: each cell its own solver, a SpikeGen of one
cell driving a synapse of another (``SpikeGen`` ``spikeOut`` ->
``Synapse::addSpike``, ``synapse/Synapse.cpp:104-113``: the spike time
plus the synapse's delay, with its weight, queued on the target's
``SimpleSynHandler``).

The solvers run in chunks no longer than the shortest delay: a spike sent
in a chunk is due, at the earliest, one delay later, after the chunk ends,
so the chunk's spikes can be queued at its end (``hs_push_events``) and the
target delivers each at the step the reference delivers it at -- the first
step whose clock time reaches spike time + delay, never the sending step
(a zero delay makes chunks of one step).  The delivery does not depend on
the chunk length.  With every cell an ``HSolve`` the chunks step them all
in one ``hs_process_group`` call; ``BatchNetwork`` does the same for the
cells of one batch (one spike read and one event push per chunk).  The
solvers keep every spike since reinit, so a run is bounded by their spike
capacity (``hs_read_spikes``/``hs_batch_read_spikes`` report an overflow).
"""
import math

import numpy as np


class Network:
    """`cells`: one solver per cell (``moose_gb300.hsolve.HSolve``, or any
    object with ``process(n)``, ``spikes()`` -> (SpikeGen indices, times)
    since reinit, and ``push_events(syn, time, weight)``); `connections`:
    (source cell, its SpikeGen, target cell, its SynChan, delay, weight)."""

    def __init__(self, cells, connections, dt):
        self.cells = list(cells)
        self.dt = float(dt)
        self.out = {}
        delays = []
        for src, gen, dst, syn, delay, weight in connections:
            if not (0 <= src < len(self.cells) and 0 <= dst < len(self.cells)):
                raise ValueError("connection (%d -> %d): no such cell" % (src, dst))
            if delay < 0:
                raise ValueError("connection (%d -> %d): negative delay" % (src, dst))
            self.out.setdefault((int(src), int(gen)), []).append((int(dst), int(syn), float(delay), float(weight)))
            delays.append(float(delay))
        # the longest chunk whose spikes are all due after it ends
        self.chunk = max(1, int(math.floor(min(delays) / self.dt * (1.0 - 1e-12)))) if delays else None
        self.seen = [0] * len(self.cells)
        self._tick = None
        try:
            from .hsolve import HSolve, Tick
            if self.cells and all(isinstance(c, HSolve) for c in self.cells):
                self._tick = Tick(self.cells)
        except ImportError:
            pass

    def reinit(self):
        """After the cells' own reinit: spikes before it are not sent."""
        self.seen = [0] * len(self.cells)

    def run(self, nsteps):
        done = 0
        while done < nsteps:
            n = nsteps - done if self.chunk is None else min(self.chunk, nsteps - done)
            if self._tick is not None:
                self._tick.process(n)
            else:
                for c in self.cells:
                    c.process(n)
            done += n
            self._send()

    def _send(self):
        queued = {}
        for i, c in enumerate(self.cells):
            gens, times = c.spikes()
            new = range(self.seen[i], len(times))
            self.seen[i] = len(times)
            for j in new:
                for dst, syn, delay, weight in self.out.get((i, int(gens[j])), ()):
                    queued.setdefault(dst, []).append((syn, float(times[j]) + delay, weight))
        for dst, ev in queued.items():
            syn, t, w = zip(*ev)
            self.cells[dst].push_events(np.array(syn, np.uint32), np.array(t), np.array(w))


class BatchNetwork:
    """The same coupling for cells stepped together in one batch
    (``moose_gb300.batch.Batch``: ``process(n)``, ``spikes()`` -> (cells,
    SpikeGens, times) since reinit, ``push_events(cells, syn, time,
    weight)``); `connections` name cells by their index in the batch.  One
    spike read and one event push per chunk, whatever the number of
    cells."""

    def __init__(self, batch, connections, dt):
        self.batch = batch
        self.dt = float(dt)
        self.out = {}
        delays = []
        for src, gen, dst, syn, delay, weight in connections:
            if delay < 0:
                raise ValueError("connection (%d -> %d): negative delay" % (src, dst))
            self.out.setdefault((int(src), int(gen)), []).append((int(dst), int(syn), float(delay), float(weight)))
            delays.append(float(delay))
        self.chunk = max(1, int(math.floor(min(delays) / self.dt * (1.0 - 1e-12)))) if delays else None
        self.seen = {}

    def reinit(self):
        self.seen = {}

    def run(self, nsteps):
        done = 0
        while done < nsteps:
            n = nsteps - done if self.chunk is None else min(self.chunk, nsteps - done)
            self.batch.process(n)
            done += n
            # every cell's spikes since reinit, each cell's in time order:
            # the new ones are those past the count already seen per cell
            cells, gens, times = self.batch.spikes()
            count, ev = {}, []
            for j in range(len(times)):
                c = int(cells[j])
                k = count.get(c, 0)
                count[c] = k + 1
                if k < self.seen.get(c, 0):
                    continue
                for dst, syn, delay, weight in self.out.get((c, int(gens[j])), ()):
                    ev.append((dst, syn, float(times[j]) + delay, weight))
            self.seen = count
            if ev:
                c, s, t, w = zip(*ev)
                self.batch.push_events(np.array(c, np.uint32), np.array(s, np.uint32), np.array(t), np.array(w))
