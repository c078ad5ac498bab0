"""Statistics of the solver's outputs, as MOOSE's ``Stats`` and ``SpikeStats``
objects compute them (``builtins/Stats.cpp``, ``builtins/SpikeStats.cpp``).

In a MOOSE script these objects sit on their own clock ticks (``Stats`` on
tick 17, ``SpikeStats`` on tick 7, after the HSolve's tick 6): a ``Stats``
requests a value (e.g. a compartment's Vm through the zombie getter) each
time its tick fires, and a ``SpikeStats`` counts the spikes that reached it
(``addSpike``) and inputs count / dt each time its tick fires.  A tick of
``k`` base steps fires at the steps whose end step is a multiple of ``k``
(``Clock::handleStep``, ``scheduling/Clock.cpp:724-775``).  The solver
records exactly those values on the device (``hs_record`` with stride
``k`` samples at the same step ends; its sample 0 is the reinit value,
which no Stats sees) and the spike times of its SpikeGens, so the same
statistics come from the recorded outputs after the run, with the
reference's arithmetic:

* ``Stats``: sum, sum of squares and count of the inputs; mean = sum / n,
  sdev = sqrt((sumsq - sum^2 / n) / n); a window of the last
  ``windowLength`` inputs (``wmean``, ``wsdev``, ``wsum``, ``wnum``; the
  window's sums run over the ring buffer in slot order, as
  ``Stats::innerWindowCalculation`` does).
* ``SpikeStats``: a Stats of count / dt per tick.
"""
import math

import numpy as np


class Stats:
    """builtins/Stats.cpp (input, mean, sdev, sum, num, window fields)."""

    def __init__(self, windowLength=0):
        self.samples = [0.0] * int(windowLength) if 0 < windowLength < 1e6 else []
        self.reinit()

    def reinit(self):
        self.sum_ = 0.0
        self.sumsq = 0.0
        self.num = 0
        self.samples = [0.0] * len(self.samples)

    def input(self, v):
        v = float(v)
        self.sum_ += v
        self.sumsq += v * v
        if self.samples:
            self.samples[self.num % len(self.samples)] = v
        self.num += 1

    @property
    def sum(self):
        return self.sum_

    @property
    def mean(self):
        return self.sum_ / self.num if self.num > 0 else 0.0

    @property
    def sdev(self):
        if self.num > 0:
            return math.sqrt((self.sumsq - self.sum_ * self.sum_ / self.num) / self.num)
        return 0.0

    def _window(self):
        wsum = wsumsq = 0.0
        n = min(len(self.samples), self.num)
        for i in range(n):
            wsum += self.samples[i]
            wsumsq += self.samples[i] * self.samples[i]
        if n > 0:
            return wsum, wsum / n, math.sqrt((wsumsq - wsum * wsum / n) / n), n
        return wsum, 0.0, 0.0, 0

    @property
    def wsum(self):
        return self._window()[0]

    @property
    def wmean(self):
        return self._window()[1]

    @property
    def wsdev(self):
        return self._window()[2]

    @property
    def wnum(self):
        return self._window()[3]


class SpikeStats(Stats):
    """builtins/SpikeStats.cpp: spikes counted between ticks, each tick
    inputs count / dt."""

    def __init__(self, windowLength=0, threshold=0.0):
        self.threshold = threshold
        super().__init__(windowLength)

    def reinit(self):
        super().reinit()
        self.num_spikes = 0
        self.fired = False

    def add_spike(self, t=0.0):
        self.num_spikes += 1

    def vm(self, v):
        """The Vm input: a spike each time Vm rises above threshold."""
        if self.fired:
            if v < self.threshold:
                self.fired = False
        elif v > self.threshold:
            self.fired = True
            self.num_spikes += 1

    def process(self, dt):
        rate = float(self.num_spikes) / dt
        self.num_spikes = 0
        self.input(rate)


def stats_of_samples(samples, windowLength=0):
    """A Stats fed the values its tick requested, in order: e.g. the trace a
    solver recorded with the Stats tick's stride, without the reinit sample
    (``trace[1:]``)."""
    s = Stats(windowLength)
    for v in np.asarray(samples, np.float64).ravel():
        s.input(v)
    return s


def spike_stats_of_times(spike_times, dt, stride, nsteps, windowLength=0):
    """A SpikeStats on a tick of `stride` base steps of `dt`, fed the spike
    times a solver recorded over `nsteps` steps.  A SpikeGen on the
    solver's tick sends its spike at the step's clock time dt x endStep
    (``SpikeGen::process``), before the SpikeStats' tick in the same step;
    the tick at end step E counts the spikes of end steps after the
    previous tick, up to E, and inputs count / (stride x dt)."""
    s = SpikeStats(windowLength)
    ends = sorted(int(round(t / dt)) for t in np.asarray(spike_times, np.float64).ravel())
    k = 0
    tick_dt = stride * dt
    for E in range(stride, nsteps + 1, stride):
        while k < len(ends) and ends[k] <= E:
            s.add_spike()
            k += 1
        s.process(tick_dt)
    return s
