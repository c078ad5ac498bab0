"""Continuous-batching serving loop over the mixed-precision batch.

Simulation requests (one cell, a number of dt steps) arrive over time.  The
loop keeps a set of running cohorts.  A cohort is a mixed-precision
``Batch`` with its own CUDA stream, whose state stays on the device between
chunks of dt steps; every cell in it stops at its own step count
(``Batch.set_stop_steps``), so one cohort holds requests of any duration.
The loop repeatedly:

  * admits waiting requests first come, first served (at most every
    ``admit_interval`` seconds, to group arrivals) while the device memory of
    the running cohorts plus the estimate for the request stays within the
    HBM budget, sets them up as a new cohort and queues its first chunk;
  * polls every cohort without waiting (``Batch.idle``): a cohort whose chunk
    has finished streams out the new soma Vm samples and spikes of its
    requests, completes the requests that reached their step count, and
    either queues its next chunk or, when all its cells are done, releases
    its memory.

Cohorts thus progress independently and their kernels run at the same time
on the GPU: a cohort's persistent kernel holds only the SMs its forests need,
the rest go to the others.  A request's latency is completion minus arrival
(queueing, setup and simulation).  A cell's result does not depend on the
cohort it runs in or on the other requests (every node's arithmetic depends
only on its own cell): the tests compare each request served in a mix with
the same request run alone.
"""
import dataclasses
import os
import time

import numpy as np

from .abi import HS_PREC_MIXED
from .batch import Batch


def configure_work_queues(n=32):
    """Ask CUDA for `n` hardware work queues (CUDA_DEVICE_MAX_CONNECTIONS,
    at most 32; 8 by default).  Kernels of different streams run at the same
    time only up to that number, so with more running cohorts than queues
    the cohorts share queues and run one after another.

    Precondition: call it before CUDA starts in the process (before the
    first call into the library or torch.cuda); afterwards the context
    keeps the number it opened with.  An existing setting in the
    environment is kept.  Returns the value in effect for a context created
    from now on."""
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", str(int(n)))
    return int(os.environ["CUDA_DEVICE_MAX_CONNECTIONS"])


@dataclasses.dataclass
class Request:
    rid: int
    cell: object            # abi.CellModel
    n_steps: int
    arrival: float = 0.0    # seconds after the start of the run


@dataclasses.dataclass
class Result:
    rid: int
    n_compt: int
    n_steps: int
    arrival: float
    admitted: float
    finished: float
    vm: np.ndarray          # soma Vm every record_stride steps; sample 0 is the reinit state
    spike_times: np.ndarray

    @property
    def latency(self):
        return self.finished - self.arrival


def estimate_bytes(cell, n_steps, record_stride):
    """Device memory a request takes in a cohort: per compartment (node
    arrays, FP64 gate states, junction nodes), per synapse and event, its
    trace and its spike buffer.  With ``cohort_overhead`` of the cohort, an
    upper bound of what ``Batch.device_bytes`` reports (checked by the
    tests)."""
    n = cell.n_compt
    samples = n_steps // record_stride + 2
    return 640 * n + 64 * len(cell.syn_compt) + 16 * len(cell.ev_time) + 8 * samples + 16384


def cohort_overhead(cell):
    """Device memory a cohort holds once whatever its size: the FP32 rate
    tables (merged 1-D table, 2-D tables), with a margin for resampling."""
    rows = max((len(g[2]) for g in cell.gates), default=0) + 2
    table = rows * 2 * len(cell.gates) * 4
    table2d = sum(np.asarray(g[4]).size * 8 for g in cell.gates2d)
    return int(1.25 * (table + table2d)) + (1 << 20)


class _Cohort:
    def __init__(self, reqs, dt, record_stride, chunk, now, tuning):
        self.reqs = reqs
        self.admitted = now
        n = len(reqs)
        self.batch = Batch([r.cell for r in reqs], dt, HS_PREC_MIXED, steps_per_launch=chunk, **tuning)
        self.stride = record_stride
        self.cap = max(r.n_steps for r in reqs) // record_stride + 2
        self.batch.record(np.arange(n), np.zeros(n, np.uint32), record_stride, self.cap)
        self.batch.set_stop_steps([r.n_steps for r in reqs])
        self.batch.reinit(dt)
        self.launched = 0                  # dt steps queued so far
        self.next_sample = 0               # first sample not streamed yet
        self.vm = [[] for _ in reqs]
        self.spikes_seen = np.zeros(n, np.int64)
        self.spikes = [[] for _ in reqs]
        self.done = np.zeros(n, bool)
        self.bytes = self.batch.device_bytes()
        self.ctas = self.batch.info()["n_ctas"]

    def launch(self, chunk):
        self.batch.process(chunk)
        self.launched += chunk

    def ready(self):
        return self.batch.idle()

    def collect(self):
        """Stream the samples and spikes of the last chunk; return the
        indices of requests that completed with it."""
        last = min(self.launched // self.stride, self.cap - 1)
        count = last - self.next_sample + 1 if last >= self.next_sample else 0
        rows, steps, counts = self.batch.poll(self.next_sample, count)
        if count:
            for i, r in enumerate(self.reqs):
                if self.done[i]:
                    continue
                k_end = min(last, r.n_steps // self.stride)     # the cell's own samples
                if k_end >= self.next_sample:
                    self.vm[i].append(rows[: k_end - self.next_sample + 1, i].copy())
            self.next_sample = last + 1
        for i in np.nonzero(counts > self.spikes_seen)[0]:
            _, t, _ = self.batch.cell_spikes(int(i), int(self.spikes_seen[i]))
            self.spikes[i].append(t)
            self.spikes_seen[i] += len(t)
        fresh = [i for i, r in enumerate(self.reqs) if not self.done[i] and steps[i] >= r.n_steps]
        for i in fresh:
            self.done[i] = True
        return fresh

    def close(self):
        self.batch.close()


class Server:
    """The serving loop.  ``budget_bytes`` bounds the device memory of the
    running cohorts; ``chunk`` is the number of dt steps a cohort advances
    between two polls of its output.  A cohort gets one CTA per request while
    the GPU's ``sms`` SMs have room; once they are taken (and with ``dense``)
    it is packed into as few CTAs as forests of about ``forest_nodes`` nodes
    need.  At most
    ``max_cohorts`` cohorts run at once (the hardware work queues of the
    context); requests that arrive meanwhile wait and start together as the
    next cohort.  An admission round makes one cohort per class of request
    present: a duration class (``duration_classes``: dt-step boundaries)
    crossed with a size class (``size_classes``: compartment-count
    boundaries).  The requests that share a cohort, and so its forests, then
    end at about the same time, and the kernel skips a forest whose cells
    have all stopped, which frees its SM.  And a launch of a cohort lasts as
    long as its slowest CTA, so a small request is not held to the step time
    of a large cell admitted beside it.  A cohort of the largest size class
    gets ``cluster_ctas`` SMs per request (a thread-block cluster assembles
    each cell, ~20 % less step latency for 5,000-10,000 compartments) while
    the GPU has that many SMs free.

    Cohorts overlap on the GPU only as far as the context's hardware work
    queues allow: call ``configure_work_queues(max_cohorts)`` before CUDA
    starts in the process."""

    def __init__(self, dt, budget_bytes=150 * 10**9, chunk=4000, record_stride=40, max_cohort=4096,
                 admit_interval=0.05, dense=True, forest_nodes=7000, max_cohorts=32, sms=152, tuning=None,
                 clock=time.perf_counter, cohort_factory=None, duration_classes=(16000, 40000),
                 size_classes=(1000, 4000), cluster_ctas=4):
        self.dt = dt
        self.budget = budget_bytes
        self.chunk = chunk
        self.stride = record_stride
        self.max_cohort = max_cohort
        self.admit_interval = admit_interval
        self.dense = dense
        self.forest_nodes = forest_nodes
        self.max_cohorts = max_cohorts
        self.sms = sms
        self.tuning = dict(tuning or {})
        self.clock = clock
        self.cohort_factory = cohort_factory or _Cohort
        self.duration_classes = tuple(sorted(duration_classes or ()))
        self.size_classes = tuple(sorted(size_classes or ()))
        self.cluster_ctas = int(cluster_ctas or 1)
        self.cohorts = []
        self.waiting = []
        self.results = []
        self.ticks = 0
        self.peak_bytes = 0

    def used_bytes(self):
        return sum(c.bytes for c in self.cohorts)

    def _class(self, r):
        """(duration class, size class) of a request."""
        return (sum(r.n_steps >= b for b in self.duration_classes),
                sum(r.cell.n_compt >= b for b in self.size_classes))

    def _admit(self, now):
        """A cohort of waiting requests of the first waiting request's
        duration class, in arrival order, within the memory budget."""
        take, est = [], 0
        used = self.used_bytes()
        if not self.waiting:
            return None
        cls = self._class(self.waiting[0])
        k = 0
        while k < len(self.waiting) and len(take) < self.max_cohort:
            r = self.waiting[k]
            if self._class(r) != cls:
                k += 1
                continue
            e = estimate_bytes(r.cell, r.n_steps, self.stride)
            if not take:
                e += cohort_overhead(r.cell)
            if used + est + e > self.budget:
                break
            take.append(self.waiting.pop(k))
            est += e
        if not take:
            return None
        tuning = dict(self.tuning)
        if "max_ctas" not in tuning:
            busy = sum(getattr(c, "ctas", 0) for c in self.cohorts)
            big = self.size_classes and cls[1] == len(self.size_classes)
            if big and self.cluster_ctas > 1 and busy + len(take) * self.cluster_ctas <= self.sms:
                # the largest cells, SMs to spare: a cluster of SMs per
                # request for the step latency
                tuning["max_ctas"] = len(take) * self.cluster_ctas
                tuning["cluster_ctas"] = self.cluster_ctas
            elif busy + len(take) <= self.sms or not self.dense:
                # room on the GPU: one CTA (one SM) per request, each runs
                # as fast as alone
                tuning["max_ctas"] = len(take)
            else:
                # the SMs are taken: as few CTAs as full forests need, each
                # SM well used
                nodes = sum(int(1.3 * r.cell.n_compt) for r in take)
                tuning["max_ctas"] = max(1, -(-nodes // self.forest_nodes))
        return self.cohort_factory(take, self.dt, self.stride, self.chunk, now, tuning)

    def run(self, requests, real_time=True, t0=None):
        """Serve `requests` (sorted by arrival); returns the results in
        completion order.  With real_time, arrivals follow the clock from t0;
        otherwise every request is available from the start."""
        pending = list(requests)
        start = self.clock() if t0 is None else t0
        last_admit = -1e30
        while pending or self.waiting or self.cohorts:
            now = self.clock() - start
            while pending and (not real_time or pending[0].arrival <= now):
                self.waiting.append(pending.pop(0))
            progressed = False
            if self.waiting and now - last_admit >= self.admit_interval and len(self.cohorts) < self.max_cohorts:
                last_admit = now
                # one cohort per class present
                for _ in range((len(self.duration_classes) + 1) * (len(self.size_classes) + 1)):
                    if not self.waiting or len(self.cohorts) >= self.max_cohorts:
                        break
                    fresh = self._admit(now)
                    if fresh is None:
                        break
                    fresh.launch(self.chunk)
                    self.cohorts.append(fresh)
                    progressed = True
            for c in list(self.cohorts):
                if not c.ready():
                    continue
                progressed = True
                done = c.collect()
                t = self.clock() - start
                for i in done:
                    r = c.reqs[i]
                    vm = np.concatenate(c.vm[i]) if c.vm[i] else np.zeros(0)
                    sp = np.concatenate(c.spikes[i]) if c.spikes[i] else np.zeros(0)
                    self.results.append(Result(r.rid, r.cell.n_compt, r.n_steps, r.arrival, c.admitted, t, vm, sp))
                if c.done.all():
                    self.cohorts.remove(c)
                    c.close()
                else:
                    c.launch(self.chunk)
            self.peak_bytes = max(self.peak_bytes, self.used_bytes())
            self.ticks += 1
            if not progressed and real_time:
                # nothing finished and nothing to admit: wait a little (until
                # the next arrival at most)
                wait = 0.0005
                if not self.cohorts and not self.waiting and pending:
                    wait = max(0.0, min(0.05, pending[0].arrival - (self.clock() - start)))
                time.sleep(wait)
        return self.results


def summarize(results, wall_s, offered_rate=None):
    """p50/p99 latency, throughput in compartment-steps/s over `wall_s`."""
    lat = np.array([r.latency for r in results])
    work = sum(r.n_compt * r.n_steps for r in results)
    out = {"requests": len(results), "wall_s": wall_s,
           "p50_latency_s": float(np.percentile(lat, 50)) if len(lat) else None,
           "p99_latency_s": float(np.percentile(lat, 99)) if len(lat) else None,
           "compartment_steps_per_s": work / wall_s if wall_s > 0 else None}
    if offered_rate is not None:
        out["offered_rate_per_s"] = offered_rate
    if len(results) >= 8:
        # queueing delay (admission minus arrival) by arrival order: a queue
        # that stays bounded keeps the last quarter's delay near the first's
        rs = sorted(results, key=lambda r: r.arrival)
        wait = np.array([r.admitted - r.arrival for r in rs])
        q = len(wait) // 4
        out["p50_queue_wait_s"] = float(np.percentile(wait, 50))
        out["p99_queue_wait_s"] = float(np.percentile(wait, 99))
        out["queue_wait_first_quarter_s"] = float(wait[:q].mean())
        out["queue_wait_last_quarter_s"] = float(wait[-q:].mean())
    return out
