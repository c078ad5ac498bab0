"""Inputs that MOOSE scripts drive a solved cell with, as the solver's own
inputs: synaptic input from ``TimeTable`` objects as queued events, and
``PulseGen`` or ``StimulusTable`` output into ``injectMsg`` as the inject
schedule.

A script drives a SynChan's synapse with a ``TimeTable``
(``builtins/TimeTable.cpp:181-205``) on tick 8: each time the tick fires,
at most one table entry whose time has come (``currTime >= t``) is sent,
with the table time ``t``; ``Synapse::addSpike`` queues it at ``t +
delay`` with the synapse's weight (``synapse/Synapse.cpp:104-113``), and
``SimpleSynHandler`` delivers it on tick 1 of the first later step whose
clock time reaches that time (``synapse/SimpleSynHandler.cpp:98-113``).
The solver delivers a queued event at the first step whose clock time
``dt x step`` reaches the event's time, so each event becomes the time of
the step the reference delivers it at: ``t + delay`` where that is later
than the step after the send, else that step's clock time exactly (the
same ``dt x step`` product the solver compares with).  The activation it
adds (weight / dt) does not depend on the time.
"""
import math

import numpy as np


def timetable_events(times, dt, nsteps, stride=1, delay=0.0, before_handler=False):
    """Queued event times for the entries `times` of one TimeTable on a tick
    of `stride` base steps of `dt`, over `nsteps` steps, into a synapse of
    the given `delay`.  On its default tick 8 the table sends after the
    handler's tick 1, so an entry reaches the synapse from the next step
    on; on tick 0 (`before_handler`) from the step it is sent in.  Entries
    the table has not sent by the end of the run are left out."""
    vec = [float(t) for t in np.asarray(times, np.float64).ravel()]
    out = []
    cur = 0
    for E in range(stride, nsteps + 1, stride):
        now = dt * E                          # Clock: currTime = dt x endStep
        if cur < len(vec) and now >= vec[cur]:
            t = vec[cur] + delay
            first = dt * (E if before_handler else E + 1)   # the first step that may deliver it
            out.append(t if t > first else first)
            cur += 1
    return np.array(out, np.float64)


def add_timetables(model, tables, dt, nsteps, stride=1, before_handler=()):
    """Queue the events of TimeTables on a model's SynChans: `tables` maps a
    SynChan index to (times, delay, weight); `before_handler` lists the
    SynChans whose table runs on tick 0.  The model's existing events are
    kept."""
    syn, tim, wts = [model.ev_syn], [model.ev_time], [model.ev_weight]
    for k, (times, delay, weight) in sorted(tables.items()):
        ev = timetable_events(times, dt, nsteps, stride, delay, before_handler=k in before_handler)
        syn.append(np.full(len(ev), k, np.uint32))
        tim.append(ev)
        wts.append(np.full(len(ev), float(weight)))
    model.ev_syn = np.concatenate(syn).astype(np.uint32)
    model.ev_time = np.concatenate(tim)
    model.ev_weight = np.concatenate(wts)
    return model


class PulseGen:
    """``device/PulseGen.cpp`` in free-run mode (trigMode 0): pulses of
    ``level[i]`` for ``width[i]`` after ``delay[i]``, ``baseLevel``
    otherwise, repeating with the reference's period; the output is kept
    from the previous call where no pulse or gap claims the phase, as
    ``PulseGen::process`` keeps ``output_``."""

    def __init__(self, level, width, delay, baseLevel=0.0):
        self.level = [float(x) for x in level]
        self.width = [float(x) for x in width]
        self.delay = [float(x) for x in delay]
        if not (len(self.level) == len(self.width) == len(self.delay)) or not self.level:
            raise ValueError("PulseGen: level, width and delay need one entry per pulse")
        self.baseLevel = float(baseLevel)
        self.output = self.baseLevel

    def reinit(self):
        self.output = self.baseLevel
        return self.output

    def process(self, t):
        w, d = self.width, self.delay
        period = w[0] + d[0]
        for i in range(1, len(w)):
            if not (w[i] > 0.0 or d[i] > 0.0):
                break
            incr = d[i] + w[i] - w[i - 1]
            if incr > 0:
                period += incr
        phase = math.fmod(t, period)
        if phase >= period:
            self.output = self.baseLevel
            return self.output
        for i in range(len(w)):
            if phase < d[i]:
                self.output = self.baseLevel
                break
            elif phase < d[i] + w[i]:
                self.output = self.level[i]
                break
            phase -= d[i]
        return self.output


class StimulusTable:
    """``builtins/StimulusTable.cpp``: the table ``vector`` spread over
    [startTime, stopTime] and read by ``TableBase::interpolate``
    (``builtins/TableBase.cpp:470-495``) at a position that advances by
    ``stepSize`` per call (accumulated), or is the clock time when
    ``stepSize`` is 0; with ``doLoop`` the position wraps every
    ``loopTime`` after ``startTime``."""

    def __init__(self, vector, startTime, stopTime, stepSize=0.0, doLoop=False, loopTime=0.0):
        self.vec = [float(v) for v in vector]
        self.start, self.stop = float(startTime), float(stopTime)
        self.stepSize, self.doLoop, self.loopTime = float(stepSize), bool(doLoop), float(loopTime)
        self.pos = 0.0

    def _interpolate(self, x):
        v, xmin, xmax = self.vec, self.start, self.stop
        if not v:
            return 0.0
        if len(v) == 1 or x < xmin or xmin >= xmax:
            return v[0]
        if x > xmax:
            return v[-1]
        xdivs = len(v) - 1
        fraction = (x - xmin) / (xmax - xmin)
        if fraction < 0:
            return v[0]
        j = int(xdivs * fraction)
        if j >= len(v) - 1:
            return v[-1]
        dx = (xmax - xmin) / xdivs
        lower = xmin + j * dx
        sub = (x - lower) / dx
        return v[j] + (v[j + 1] - v[j]) * sub

    def reinit(self):
        self.pos = 0.0
        return self._interpolate(self.pos)

    def process(self, t):
        if self.stepSize > 0:
            self.pos += self.stepSize
        else:
            self.pos = t
        x = self.pos
        if self.doLoop and self.pos > self.start + self.loopTime:
            i = math.floor((self.pos - self.start) / self.loopTime)
            x = self.pos - self.loopTime * i
        return self._interpolate(x)


def add_pulsegen(model, compt, pulse, dt, nsteps, stride=1, after_solver=False):
    """A PulseGen's ``output`` into compartment `compt`'s ``injectMsg``, as
    the model's inject schedule.  The PulseGen runs on a tick of `stride`
    steps and its output reaches a step's right-hand side through
    ``HSolve::addInject`` (``injectVarying``, used and cleared by the next
    matrix update, ``hsolve/HSolveActive.cpp:118-126``): on a tick before
    the solver's tick 6 (tick 0, the default) the same step's, on a later
    tick (`after_solver`) the next step's.  The value it sends at reinit
    stays in ``injectVarying`` until the first step uses it.  The schedule sets
    the compartment's basal inject each step to what the reference adds:
    (the step's messages) + (the compartment's inject), in that order.
    The model must have no other schedule entries for `compt`."""
    base = float(model.inject[compt])
    if np.any(model.stim_compt == compt):
        raise ValueError("add_pulsegen: compartment %d already has scheduled injects" % compt)
    pending = pulse.reinit()              # sent at reinit, kept until step 0
    steps, vals = [], []
    prev = base
    for s in range(nsteps):
        E = s if after_solver else s + 1      # the end step whose tick sent this step's value
        varying = pending
        pending = 0.0
        if E >= 1 and E % stride == 0:
            varying = varying + pulse.process(dt * E)   # Clock: currTime = dt x endStep
        v = varying + base if varying != 0.0 else base
        if v != prev or s == 0:
            steps.append(s)
            vals.append(v)
            prev = v
    model.stim_step = np.concatenate([model.stim_step, np.array(steps, np.uint32)])
    model.stim_compt = np.concatenate([model.stim_compt, np.full(len(steps), compt, np.uint32)])
    model.stim_value = np.concatenate([model.stim_value, np.array(vals, np.float64)])
    order = np.lexsort((model.stim_compt, model.stim_step))
    model.stim_step, model.stim_compt, model.stim_value = (model.stim_step[order], model.stim_compt[order],
                                                           model.stim_value[order])
    return model


# any source with reinit() and process(t) (PulseGen, StimulusTable) into injectMsg
add_injector = add_pulsegen
