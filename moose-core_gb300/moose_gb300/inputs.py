"""Synaptic input from MOOSE ``TimeTable`` objects, as queued events of the
solver.

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
import numpy as np


def timetable_events(times, dt, nsteps, stride=1, delay=0.0):
    """Queued event times for the entries `times` of one TimeTable on a tick
    of `stride` base steps of `dt`, over `nsteps` steps, into a synapse of
    the given `delay`.  Entries the table has not sent by the end of the
    run are left out."""
    vec = [float(t) for t in np.asarray(times, np.float64).ravel()]
    out = []
    cur = 0
    for E in range(stride, nsteps + 1, stride):
        now = dt * E                          # Clock: currTime = dt x endStep
        if cur < len(vec) and now >= vec[cur]:
            t = vec[cur] + delay
            first = dt * (E + 1)              # the next step's clock time
            out.append(t if t > first else first)
            cur += 1
    return np.array(out, np.float64)


def add_timetables(model, tables, dt, nsteps, stride=1):
    """Queue the events of TimeTables on a model's SynChans: `tables` maps a
    SynChan index to (times, delay, weight).  The model's existing events
    are kept."""
    syn, tim, wts = [model.ev_syn], [model.ev_time], [model.ev_weight]
    for k, (times, delay, weight) in sorted(tables.items()):
        ev = timetable_events(times, dt, nsteps, stride, delay)
        syn.append(np.full(len(ev), k, np.uint32))
        tim.append(ev)
        wts.append(np.full(len(ev), float(weight)))
    model.ev_syn = np.concatenate(syn).astype(np.uint32)
    model.ev_time = np.concatenate(tim)
    model.ev_weight = np.concatenate(wts)
    return model
