#!/usr/bin/env python3
"""bench.py -- HSolve compartment-steps/s on GB300.

Workload (one GPU): the 4,096-cell mixed-precision batch -- seeded synthetic
cells with log-uniform 50..5,000 compartments, junctions of up to 4 children,
HH Na/K + Ca(HVA) + K(Ca) (HHChannel2D on Vm x Ca) + CaConc on every
compartment, 200 dual-exponential SynChans per cell driven by 5 Hz Poisson
trains, a somatic step current, dt = 25 us.  One bench step is one chunk of
--chunk (default 200) dt steps of all cells.  Data are synthetic (seeded);
the working set (~1 GB of state) is larger than L2, so no L2 flush is needed.

The JSON line carries:
  value      mixed-precision batch, device-timed (CUDA events on the batch's
             stream), inputs resident on the GPU;
  e2e        the same through the C ABI with host buffers: every step copies
             the somatic inject of every cell from pinned host memory and
             reads back the somatic Vm trace of the chunk;
  fp64_dropin the plain FP64 drop-in (one HSolve instance per cell, one CTA
             each) on a sample of the same cells, and the ratio to `value`;
  single_cell the FP64 drop-in on the single-cell case (soma + 200-compartment
             HH cable, 0.5 s), next to the same cell on one host core;
  fp64_batch the FP64 batch (one warp per cell, the drop-in's arithmetic,
             bit-identical results) on all cells of the workload;
  accuracy   max |dVm| (soma every dt step, every compartment every 1,000
             steps) and spike-time shift of the mixed batch against the FP64
             batch (bit-identical to the reference HSolve) on 256 of the
             cells for the full 1 s (--accuracy-full: all 4,096 cells);
  config2    the 256-cell workload as written: every cell its own FP64
             drop-in HSolve, beside the CPU restatement on the same cells;
  roofline   the stepping kernel against the measured HBM copy bandwidth;
  cpu_baseline the CPU restatement of HSolve (the oracle) on the host cores;
  config.autotuned  the packing and launch shape the autotuner picked.
  serving    the serving loop (continuous batching under a 150 GB budget)
             on Poisson arrivals of the serving workload: p50/p99 latency
             and compartment-steps/s at the offered 2,000 requests/s over a
             bounded window, and at a low rate (10 requests/s).
With --impl reference the line is the CPU HSolve on all host cores instead.
With --gpus N (torchrun) every rank runs its own replica ("replicas only").
"""
import argparse
import json
import math
import multiprocessing as mp
import os
import subprocess
import sys
import tempfile
import threading
import time

# concurrent kernels of the serving loop's cohorts need more hardware work
# queues than the default 8 (set before CUDA starts in this process)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "moose-core_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

DT = 25e-6
CONFIG = 4
SEED = 1


# ---------------------------------------------------------------------------
# CPU side: the oracle (CPU restatement of HSolve), one process per core

def _cpu_worker(conn, cell_ids, n_cells, t_end, config=CONFIG):
    import numpy as np  # noqa: F401
    from moose_gb300 import models
    from oracle import OracleCell
    sizes, _, _ = models.population_sizes(config, SEED, n_cells)
    kca = models.kca_2d_tables()
    cells = [models.make_cell(config, SEED, i, t_end=t_end, kca_tables=kca, sizes=sizes) for i in cell_ids]
    oc = []
    for m in cells:
        o = OracleCell(m, DT)
        o.reinit(DT)
        oc.append(o)
    ncomp = sum(m.n_compt for m in cells)
    conn.send(("ready", ncomp))
    while True:
        msg = conn.recv()
        if msg is None:
            break
        t0 = time.perf_counter()
        for o in oc:
            o.step(msg)
        conn.send(("done", time.perf_counter() - t0))


class CpuPool:
    """Cells of the workload split over `workers` processes (LPT on size)."""

    def __init__(self, cell_ids, n_cells, workers, t_end, config=CONFIG):
        from moose_gb300 import models
        sizes, _, _ = models.population_sizes(config, SEED, n_cells)
        groups = [[] for _ in range(workers)]
        load = [0] * workers
        for i in sorted(cell_ids, key=lambda k: -sizes[k]):
            w = load.index(min(load))
            groups[w].append(i)
            load[w] += int(sizes[i])
        ctx = mp.get_context("spawn")
        self.conns, self.procs = [], []
        for g in groups:
            if not g:
                continue
            a, b = ctx.Pipe()
            p = ctx.Process(target=_cpu_worker, args=(b, g, n_cells, t_end, config), daemon=True)
            p.start()
            self.conns.append(a)
            self.procs.append(p)
        self.ncomp = sum(c.recv()[1] for c in self.conns)
        self.workers = len(self.conns)

    def step(self, n):
        for c in self.conns:
            c.send(n)
        return max(c.recv()[1] for c in self.conns)

    def close(self):
        for c in self.conns:
            c.send(None)
        for p in self.procs:
            p.join(timeout=10)


# ---------------------------------------------------------------------------
# clocks during the timed region

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + self.FIELDS,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait(timeout=10)
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.count(",") >= 6]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
            except ValueError:
                continue
            for k, name in enumerate(names):
                if r[3 + k].strip().lower() == "active":
                    reasons.add(name)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx,
                "samples": len(sm), "reasons": sorted(reasons)}


def _traffic_from_profiles(layout):
    """DRAM bytes per compartment-step of the stepping kernel from the
    committed ncu summary, for the forest layout the batch runs with:
    "shared" (forests eliminated in shared memory) or "global" (merged small
    forests eliminated in global memory).  None if there is no figure."""
    path = os.path.join(ROOT, "profiles", "hsForestStepMixed_4096cells.md")
    if not os.path.exists(path):
        return None
    key = "dram_bytes_per_compartment_step_%s:" % layout
    for line in open(path):
        if line.startswith(key):
            try:
                return float(line.split(":", 1)[1])
            except ValueError:
                return None
    return None


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------

def run_reference(args, rank, world):
    """The CPU HSolve (oracle port) on every host core, on bounded samples of
    the workload: each step advances a fixed subset of cells by --ref-chunk dt."""
    if rank != 0:
        return None
    workers = os.cpu_count() or 1
    ids = list(range(0, args.cells, max(1, args.cells // args.ref_cells)))[: args.ref_cells]
    t_end = (args.warmup + args.steps + 2) * args.ref_chunk * DT
    pool = CpuPool(ids, args.cells, workers, t_end)
    for _ in range(args.warmup):
        pool.step(args.ref_chunk)
    total = 0.0
    for _ in range(args.steps):
        total += pool.step(args.ref_chunk)
    pool.close()
    value = pool.ncomp * args.ref_chunk * args.steps / total
    sample = "%d of %d cells (%d compartments) x %d dt steps per step, %d processes" % (
        len(ids), args.cells, pool.ncomp, args.ref_chunk, pool.workers)
    return {"metric": "compartment-steps/s", "impl": "reference", "value": value,
            "unit": "compartment-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": "hsolve_4096cells_mixed_syn200", "cells": args.cells, "dt_s": DT,
                       "chunk_dt_steps": args.ref_chunk},
            "cpu_baseline": {"value": value, "unit": "compartment-steps/s", "cores": pool.workers,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "compartment-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def run_serving(args, capacity=None):
    """The serving loop on Poisson arrivals of the serving workload (cells of
    100..10,000 compartments, 0.1..2 s, step current or 50..500 synapses),
    150 GB budget: once at the offered rate over a bounded window (the loop is
    overloaded there: each request carries ~9e7 compartment-steps), once at a
    low rate.  Requests are generated before the clock starts."""
    import numpy as np
    from moose_gb300 import models, serve
    kca = models.kca_2d_tables()
    out = {"workload": "serving: Poisson arrivals, cells log-uniform 100..10,000 compartments, 0.1..2 s at 25 us, "
                       "step current 0.1..1 nA or 50..500 Poisson synapses at 5 Hz, mixed precision",
           "budget_bytes": args.serve_budget, "chunk_dt_steps": args.serve_chunk,
           "admit_interval_s": args.serve_admit}
    rid = 0
    runs = [("offered", args.serve_rate, args.serve_window),
            ("low_rate", args.serve_rate_low, args.serve_window_low)]
    if capacity:
        # the rate the loop sustains: a fraction of its capacity, the batch's
        # compartment-steps/s over the mean work of a serving request
        mean_work = float(np.mean([a * b for a, b in (models.serving_request_work(SEED, 10**6 + k, DT)
                                                      for k in range(4000))]))
        rate = round(args.serve_load * capacity / mean_work, 1)
        out["capacity_requests_per_s"] = capacity / mean_work
        out["mean_request_compartment_steps"] = mean_work
        runs.append(("sustained", rate, args.serve_window_sustained))
    for name, rate, window in runs:
        rng = np.random.default_rng([SEED, 77, int(rate)])
        t, arrivals = 0.0, []
        while True:
            t += rng.exponential(1.0 / rate)
            if t > window:
                break
            arrivals.append(t)
        reqs = []
        for a in arrivals:
            cell, steps = models.serving_request(SEED, rid, DT, kca)
            reqs.append(serve.Request(rid, cell, steps, arrival=a))
            rid += 1
        srv = serve.Server(DT, budget_bytes=args.serve_budget, chunk=args.serve_chunk, admit_interval=args.serve_admit)
        t0 = time.perf_counter()
        res = srv.run(reqs)
        wall = time.perf_counter() - t0
        summ = serve.summarize(res, wall, offered_rate=rate)
        summ.update({"arrival_window_s": window, "peak_device_bytes": srv.peak_bytes, "ticks": srv.ticks,
                     "mean_compartments": float(np.mean([r.n_compt for r in res])) if res else None,
                     "mean_dt_steps": float(np.mean([r.n_steps for r in res])) if res else None})
        out[name] = summ
    return out


def _probe_cell(job):
    """CPU conditioning check of one workload cell (spawned process): the
    FP64 oracle against itself with only its gate increments in FP32 (the
    gating precision of the mixed solver), over the same steps; returns the
    soma's max |dVm|, the spike-time shift and whether the counts agree."""
    import numpy as np
    from moose_gb300 import models
    from oracle import OracleCell
    config, cell, n_cells, nsteps = job
    sizes, _, _ = models.population_sizes(config, SEED, n_cells)
    m = models.make_cell(config, SEED, cell, t_end=nsteps * DT + 0.01, sizes=sizes)
    out = []
    for probe in (False, True):
        o = OracleCell(m, DT)
        o.set_f32_gate_increments(probe)
        o.reinit(DT)
        soma = np.empty(nsteps + 1)
        soma[0] = o.vm()[0]
        for k in range(nsteps):
            o.step(1)
            soma[k + 1] = o.vm()[0]
        out.append((soma, np.sort(o.spikes()[1])))
    (sa, ta), (sb, tb) = out
    eq = len(ta) == len(tb)
    return (cell, float(np.abs(sa - sb).max()), float(np.abs(ta - tb).max()) if eq and len(ta) else 0.0, eq)


def compare_mixed_fp64(cells, nsteps, chunk, ids=None, config=CONFIG, n_cells=None):
    """Accuracy of the mixed-precision batch against the FP64 batch (every
    cell bit-identical to the FP64 drop-in, itself bit-identical to the
    reference HSolve where no libm call differs): both batches step the same
    cells side by side (their own streams); the soma Vm of every cell is
    compared at every dt step, every compartment's Vm at the end of every
    chunk of `chunk` steps, and the spike trains at the end.

    Each cell over the bar (0.1 mV, 0.05 ms, equal counts) is then checked
    for conditioning on the host cores: when the FP64 oracle with only its
    gate increments in FP32 already leaves the bar on that cell, the cell is
    ill-conditioned for FP32 gating (the precision split the mixed solver is
    asked for) and is reported as such; the others would be defects."""
    import numpy as np
    from moose_gb300.abi import HS_PREC_FP64, HS_PREC_MIXED
    from moose_gb300.batch import Batch
    n = len(cells)
    ids = list(range(n)) if ids is None else list(ids)
    f = Batch(cells, DT, HS_PREC_FP64)
    mx = Batch(cells, DT, HS_PREC_MIXED)
    somas = np.zeros(n, np.uint32)
    for bb in (f, mx):
        bb.record(np.arange(n), somas, 1, nsteps + 1)
        bb.reinit(DT)
    off = np.concatenate([[0], np.cumsum([m.n_compt for m in cells])[:-1]])
    soma_dv = np.zeros(n)
    all_dv = np.zeros(n)
    done = 0
    t0 = time.perf_counter()
    wf = np.empty((chunk + 1, n))
    wm = np.empty((chunk + 1, n))
    while done < nsteps:
        k = min(chunk, nsteps - done)
        f.process(k)
        mx.process(k)
        f.sync()
        mx.sync()
        f.trace_window(done, k + 1, wf[:k + 1])
        mx.trace_window(done, k + 1, wm[:k + 1])
        soma_dv = np.maximum(soma_dv, np.abs(wf[:k + 1] - wm[:k + 1]).max(axis=0))
        all_dv = np.maximum(all_dv, np.maximum.reduceat(np.abs(f.read_all("Vm") - mx.read_all("Vm")), off))
        done += k
    wall = time.perf_counter() - t0
    cf, _, sf = f.spikes()
    cm, _, sm = mx.spikes()
    shift = np.zeros(n)
    equal = np.ones(n, bool)
    for i in range(n):
        a, b = np.sort(sf[cf == i]), np.sort(sm[cm == i])
        if len(a) != len(b):
            equal[i] = False
        elif len(a):
            shift[i] = float(np.abs(a - b).max())
    f.close()
    mx.close()
    dv = np.maximum(soma_dv, all_dv)
    over = [i for i in range(n) if dv[i] > 1e-4 or shift[i] > 5e-5 or not equal[i]]
    # conditioning of the cells over the bar, on the host cores
    ill = set()
    probes = []
    if over:
        ctx = mp.get_context("spawn")
        jobs = [(config, ids[i], n_cells or len(cells), nsteps) for i in over]
        with ctx.Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
            probes = pool.map(_probe_cell, jobs, chunksize=1)
        for (cell, pdv, psh, peq), i in zip(probes, over):
            if pdv > 1e-4 or psh > 5e-5 or not peq:
                ill.add(i)
    well = [i for i in range(n) if i not in ill]
    ncomp = sum(m.n_compt for m in cells)
    wdv = float(dv[well].max()) if well else None
    wsh = float(shift[well].max()) if well else None
    return {"max_abs_dVm_V": float(dv.max()), "max_abs_dVm_soma_every_step_V": float(soma_dv.max()),
            "max_abs_dVm_all_compartments_chunk_ends_V": float(all_dv.max()), "worst_cell": int(ids[int(dv.argmax())]),
            "max_spike_shift_s": float(shift.max()), "spike_counts_equal": bool(equal.all()),
            "cells_with_unequal_counts": int((~equal).sum()), "spikes": int(len(sf)),
            "cells": n, "compartments": ncomp, "dt_steps": nsteps, "chunk_dt_steps": chunk,
            "bounds": {"dVm_V": 1e-4, "spike_shift_s": 5e-5},
            "cells_over_bar": [{"cell": int(ids[i]), "max_abs_dVm_V": float(dv[i]), "spike_shift_s": float(shift[i]),
                                "counts_equal": bool(equal[i]),
                                "fp64_oracle_with_f32_gate_increments": {"max_abs_dVm_soma_V": p[1],
                                                                         "spike_shift_s": p[2],
                                                                         "counts_equal": p[3]}}
                               for i, p in zip(over, probes)],
            "ill_conditioned_cells": len(ill),
            "well_conditioned": {"cells": len(well), "max_abs_dVm_V": wdv, "max_spike_shift_s": wsh,
                                 "spike_counts_equal": bool(equal[well].all()) if well else None,
                                 "within_bounds": bool(well and wdv <= 1e-4 and wsh <= 5e-5
                                                       and equal[well].all())},
            "within_bounds_all_cells": bool(dv.max() <= 1e-4 and shift.max() <= 5e-5 and equal.all()),
            "wall_s": wall,
            "compared": "mixed batch vs FP64 batch: soma Vm every dt step, every compartment's Vm at every "
                        "chunk end, spike times and counts of every cell; a cell over the bar is "
                        "ill-conditioned when the FP64 oracle with only FP32 gate increments also leaves it"}


def run_accuracy_full(args):
    """The whole synaptic workload (every cell, the full 1 s) through
    compare_mixed_fp64; prints one JSON line."""
    import torch
    from moose_gb300 import models
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    kca = models.kca_2d_tables()
    sizes, _, _ = models.population_sizes(CONFIG, SEED, args.cells)
    t_end = args.acc_steps * DT + 0.01
    cells = [models.make_cell(CONFIG, SEED, i, t_end=t_end, kca_tables=kca, sizes=sizes) for i in range(args.cells)]
    out = compare_mixed_fp64(cells, args.acc_steps, args.chunk, n_cells=args.cells)
    out["workload"] = "hsolve_4096cells_mixed_syn200" if args.cells == 4096 else "%d cells" % args.cells
    return out


def run_config2(args, cpu_pool):
    """The 256-cell workload as written: every cell its own FP64 drop-in
    HSolve (one CTA, its own stream; all cells queued before any waits),
    --config2-steps dt steps, wall-clocked; beside the CPU HSolve restatement
    on the same cells on the host cores."""
    from moose_gb300 import models
    from moose_gb300.hsolve import HSolve, process_group
    n_cells = 256
    sizes, _, _ = models.population_sizes(2, SEED, n_cells)
    kca = models.kca_2d_tables()
    t_end = (args.config2_steps + 50) * DT
    cells = [models.make_cell(2, SEED, i, t_end=t_end, kca_tables=kca, sizes=sizes) for i in range(n_cells)]
    hs = []
    for m in cells:
        h = HSolve(m, dt=DT)
        h.target = m.seed
        h.reinit(DT)
        hs.append(h)
    for h in hs:
        h.process(20)
    for h in hs:
        h.sync()
    t0 = time.perf_counter()
    for h in hs:
        h.process(args.config2_steps)
    for h in hs:
        h.sync()
    wall = time.perf_counter() - t0
    # the same solvers stepped together, one hs_process_group call (one
    # launch per cluster size, a CTA or cluster per solver) in place of 256
    # hs_process calls
    process_group(hs, 20)
    for h in hs:
        h.sync()
    t0 = time.perf_counter()
    process_group(hs, args.config2_steps)
    for h in hs:
        h.sync()
    wall_g = time.perf_counter() - t0
    for h in hs:
        h.close()
    ncomp = int(sum(m.n_compt for m in cells))
    out = {"workload": "256 cells, binary branching, 100..1,000 compartments, HH + Ca(HVA) + K(Ca) HHChannel2D + "
                       "CaConc, each its own FP64 drop-in HSolve", "cells": n_cells, "compartments": ncomp,
           "dt_steps": args.config2_steps, "wall_s": wall, "value": ncomp * args.config2_steps / wall,
           "unit": "compartment-steps/s",
           "group": {"call": "hs_process_group over the 256 solvers", "wall_s": wall_g,
                     "value": ncomp * args.config2_steps / wall_g}}
    if cpu_pool is not None:
        tcpu = cpu_pool.step(args.config2_cpu_steps)
        cv = cpu_pool.ncomp * args.config2_cpu_steps / tcpu
        out["cpu_baseline"] = {"value": cv, "unit": "compartment-steps/s", "cores": cpu_pool.workers,
                               "kind": "port", "sample": "all 256 cells x %d dt steps" % args.config2_cpu_steps}
        out["gpu_over_cpu"] = out["value"] / cv
        out["group"]["gpu_over_cpu"] = out["group"]["value"] / cv
    return out


def run_ours(args, rank, world, cpu_pool):
    import numpy as np
    import torch
    from moose_gb300 import models
    from moose_gb300.abi import HS_PREC_FP64, HS_PREC_MIXED
    from moose_gb300.batch import Batch
    from moose_gb300.hsolve import HSolve, process_group
    from moose_gb300.perf import algorithmic_bytes
    from moose_gb300.replicas import barrier, job_throughput, max_over_ranks

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    total_steps = (args.warmup + 2 * args.steps + 4) * args.chunk
    t_end = total_steps * DT
    kca = models.kca_2d_tables()
    sizes, _, _ = models.population_sizes(CONFIG, SEED, args.cells)
    cells = [models.make_cell(CONFIG, SEED, i, t_end=t_end, kca_tables=kca, sizes=sizes)
             for i in range(args.cells)]
    ncomp = sum(m.n_compt for m in cells)
    b = Batch(cells, DT, HS_PREC_MIXED, steps_per_launch=args.steps_per_launch,
              forest_nodes=args.forest_nodes, elim_warps=args.elim_warps)
    tuned = None
    if not args.no_autotune:
        from moose_gb300.autotune import autotune
        tuned = autotune(b, DT, steps=200, warmup=50)
    spl = b.info()["steps_per_launch"]
    stride = 10
    cap = total_steps // stride + 2
    somas = np.zeros(args.cells, np.uint32)
    b.record(np.arange(args.cells), somas, stride, cap)
    b.inject_targets(np.arange(args.cells), somas)
    b.reinit(DT)
    stream = torch.cuda.ExternalStream(b.stream())
    inj_host = torch.empty(args.cells, dtype=torch.float64).pin_memory()
    inj_values = np.array([m.inject[0] for m in cells])
    trace_host = torch.empty((args.chunk // stride, args.cells), dtype=torch.float64).pin_memory()

    # warm-up
    for _ in range(args.warmup):
        b.process(args.chunk)
    b.sync()
    b.kernel_time()
    # device-timed throughput, inputs resident
    barrier(local)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        b.process(args.chunk)
    ev1.record(stream)
    b.sync()
    torch.cuda.synchronize()
    clk = clocks.stop()
    dev_ms = ev0.elapsed_time(ev1)
    k_ms, k_n = b.kernel_time()
    # end to end through the C ABI: inject in from pinned memory, trace out
    barrier(local)
    done = b.info()
    first = (args.warmup + args.steps) * args.chunk // stride + 1
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(args.steps):
        inj_host.copy_(torch.from_numpy(inj_values * (1.0 + 0.01 * (k % 3))))
        b.set_inject(inj_host)
        b.process(args.chunk)
        b.trace_window(first, args.chunk // stride, trace_host)
        first += args.chunk // stride
    e1.record(stream)
    b.sync()
    e2e_ms = e0.elapsed_time(e1)
    e2e_wall = time.perf_counter() - t0
    e2e_ms = max(e2e_ms, e2e_wall * 1e3)
    del done

    dev_ms = max_over_ranks(dev_ms, "cuda")
    e2e_ms = max_over_ranks(e2e_ms, "cuda")
    value = job_throughput(ncomp * args.chunk * args.steps, dev_ms / 1e3, world)
    e2e_value = job_throughput(ncomp * args.chunk * args.steps, e2e_ms / 1e3, world)

    out = None
    if rank == 0:
        peak, peak_kind = _peaks()
        bytes_step, bpc = algorithmic_bytes(cells, HS_PREC_MIXED)
        achieved = bytes_step * spl / (k_ms / 1e3) / 1e9 if k_ms > 0 else None
        info = b.info()
        layout = "global" if info["n_shared_forests"] == 0 else "shared"
        tpc = _traffic_from_profiles(layout)
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak if achieved else None,
                "traffic": tpc * ncomp * spl if tpc else None,
                "traffic_layout": layout,
                "kernel": "hsForestStepMixed", "algorithmic_bytes_per_compartment_step": round(bpc, 1),
                "launch_ms": k_ms, "launches_timed": k_n, "peak_source": peak_kind}
        # plain FP64 drop-in on a sample of the same cells: one HSolve per cell
        dropin = None
        if not args.skip_dropin:
            ids = list(range(0, args.cells, max(1, args.cells // args.dropin_cells)))[: args.dropin_cells]
            hs = []
            for i in ids:
                h = HSolve(cells[i], dt=DT)
                h.target = cells[i].seed
                h.reinit(DT)
                hs.append(h)
            for h in hs:
                h.process(20)
            for h in hs:
                h.sync()
            t0 = time.perf_counter()
            for h in hs:
                h.process(args.dropin_steps)
            for h in hs:
                h.sync()
            wall = time.perf_counter() - t0
            process_group(hs, 20)
            for h in hs:
                h.sync()
            t0 = time.perf_counter()
            process_group(hs, args.dropin_steps)
            for h in hs:
                h.sync()
            wall_g = time.perf_counter() - t0
            nc = sum(cells[i].n_compt for i in ids)
            dv = nc * args.dropin_steps / wall
            dropin = {"value": dv, "unit": "compartment-steps/s",
                      "sample": "%d of %d cells as separate FP64 HSolve instances (one stream each), %d dt steps"
                                % (len(ids), args.cells, args.dropin_steps),
                      "mixed_batch_over_fp64_dropin": value / world / dv,
                      "group": {"call": "hs_process_group over the same instances",
                                "value": nc * args.dropin_steps / wall_g}}
            for h in hs:
                h.close()
        # the FP64 batch (warp per cell, the drop-in's arithmetic) on the same workload
        fp64b = None
        if not args.skip_fp64_batch:
            f = Batch(cells, DT, HS_PREC_FP64, steps_per_launch=100)
            f.reinit(DT)
            f.process(20)
            f.sync()
            f.kernel_time()
            t0 = time.perf_counter()
            f.process(args.fp64_batch_steps)
            f.sync()
            wall = time.perf_counter() - t0
            fms, fn = f.kernel_time()
            fv = ncomp * args.fp64_batch_steps / wall
            fp64b = {"value": fv, "unit": "compartment-steps/s", "cells": args.cells,
                     "dt_steps": args.fp64_batch_steps, "kernel_ms_per_launch": fms,
                     "mixed_batch_over_fp64_batch": value / world / fv,
                     "fp64_batch_over_fp64_dropin": (fv / dropin["value"]) if dropin else None}
            f.close()
        acc = None
        if not args.skip_accuracy:
            ids = list(range(0, args.cells, max(1, args.cells // args.acc_cells)))[: args.acc_cells]
            t_acc = args.acc_steps * DT + 0.01      # synaptic trains and stimulus cover the whole run
            acc_cells = [models.make_cell(CONFIG, SEED, i, t_end=t_acc, kca_tables=kca, sizes=sizes) for i in ids]
            acc = compare_mixed_fp64(acc_cells, args.acc_steps, args.acc_chunk, ids=ids, n_cells=args.cells)
            del acc_cells
            acc["sample"] = ("%d of %d cells (every %d-th), %d dt steps (%.2f s)"
                             % (len(ids), args.cells, max(1, args.cells // args.acc_cells), args.acc_steps,
                                args.acc_steps * DT))
        # the single-cell drop-in case: soma + 200-compartment HH cable, 0.5 s
        single = None
        n1 = 20000
        if not args.skip_single:
            m1 = models.config1_cell()
            h = HSolve(m1, dt=DT)
            h.target = m1.seed
            h.reinit(DT)
            h.process(200)
            h.sync()
            h.reinit(DT)
            t0 = time.perf_counter()
            h.process(n1)
            h.sync()
            g_s = time.perf_counter() - t0
            # zombie field access between steps, as a script reading every
            # compartment's Vm after each step does: one step, then all reads
            comps = [h.compartment(i) for i in range(m1.n_compt)]
            t0 = time.perf_counter()
            for _ in range(20):
                h.process(1)
                for c in comps:
                    c.Vm
            f_s = time.perf_counter() - t0
            h.close()
            single = {"workload": "single cell: soma + 200-compartment HH cable (Na m3h, K n4), 20,000 dt steps "
                                  "of 25 us (0.5 s), FP64 drop-in through hs_process", "wall_s": g_s,
                      "value": m1.n_compt * n1 / g_s, "unit": "compartment-steps/s",
                      "us_per_step": g_s / n1 * 1e6,
                      "step_and_read_all_vm_us": f_s / 20 * 1e6,
                      "field_access": "one dt step then Vm of all %d compartments through hs_get_field, "
                                      "from Python" % m1.n_compt}
        cpu = None
        if cpu_pool is not None:
            tcpu = cpu_pool.step(args.cpu_chunk)
            tcpu += cpu_pool.step(args.cpu_chunk)
            cv = cpu_pool.ncomp * 2 * args.cpu_chunk / tcpu
            cpu = {"value": cv, "unit": "compartment-steps/s", "cores": cpu_pool.workers, "kind": "port",
                   "sample": "%d compartments of the workload's cells x %d dt steps in %d processes"
                             % (cpu_pool.ncomp, 2 * args.cpu_chunk, cpu_pool.workers)}
            if single is not None:
                # the same single cell on one host core (the CPU HSolve restatement)
                from oracle import OracleCell
                m1 = models.config1_cell()
                oc = OracleCell(m1, DT)
                oc.reinit(DT)
                t0 = time.perf_counter()
                oc.step(n1)
                c_s = time.perf_counter() - t0
                cpu["single_cell"] = {"wall_s": c_s, "value": m1.n_compt * n1 / c_s, "cores": 1,
                                      "sample": "the single-cell workload, all 20,000 dt steps"}
                single["gpu_over_cpu_1core"] = c_s / single["wall_s"]
        cfg2 = None
        if not args.skip_config2:
            cfg2 = run_config2(args, args.config2_pool)
        launches = args.steps * math.ceil(args.chunk / spl)
        out = {"metric": "compartment-steps/s", "value": value, "unit": "compartment-steps/s",
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "mixed (f32 channels, f64 solve)",
               "data": "synthetic (seeded cells; working set larger than L2, no flush)",
               "config": {"workload": "hsolve_4096cells_mixed_syn200", "cells": args.cells,
                          "compartments": ncomp, "dt_s": DT, "chunk_dt_steps": args.chunk,
                          "steps_per_launch": spl, "threads_per_cta": b.info()["threads_per_cta"],
                          "ctas": b.info()["n_ctas"], "autotuned": tuned,
                          "synchans_per_cell": 200, "parallelism": "replicas"},
               "e2e": {"value": e2e_value, "unit": "compartment-steps/s",
                       "h2d_bytes_per_step": args.cells * 8,
                       "d2h_bytes_per_step": (args.chunk // stride) * args.cells * 8},
               "roofline": roof, "cpu_baseline": cpu, "fp64_dropin": dropin, "fp64_batch": fp64b,
               "accuracy": acc, "single_cell": single, "config2": cfg2,
               "clocks": clk, "gpu_launches": launches}
        if not args.skip_serving:
            out["serving"] = run_serving(args, capacity=value / world)
    b.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cells", type=int, default=4096)
    ap.add_argument("--chunk", type=int, default=200, help="dt steps per bench step")
    ap.add_argument("--steps-per-launch", type=int, default=0)
    ap.add_argument("--forest-nodes", type=int, default=0, help="mixed batch forest size (0: one cell per forest)")
    ap.add_argument("--elim-warps", type=int, default=0, help="mixed batch eliminator warps (0: default)")
    ap.add_argument("--dropin-cells", type=int, default=128)
    ap.add_argument("--dropin-steps", type=int, default=200)
    ap.add_argument("--acc-cells", type=int, default=256)
    ap.add_argument("--acc-steps", type=int, default=40000)
    ap.add_argument("--acc-chunk", type=int, default=1000, help="dt steps between full-state comparisons")
    ap.add_argument("--accuracy-full", action="store_true",
                    help="only the accuracy comparison, on every cell of the workload for --acc-steps")
    ap.add_argument("--config2-steps", type=int, default=2000)
    ap.add_argument("--config2-cpu-steps", type=int, default=200)
    ap.add_argument("--skip-config2", action="store_true")
    ap.add_argument("--cpu-cells", type=int, default=128)
    ap.add_argument("--cpu-chunk", type=int, default=400)
    ap.add_argument("--ref-cells", type=int, default=128)
    ap.add_argument("--ref-chunk", type=int, default=200)
    ap.add_argument("--skip-dropin", action="store_true")
    ap.add_argument("--skip-accuracy", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-serving", action="store_true")
    ap.add_argument("--skip-fp64-batch", action="store_true")
    ap.add_argument("--skip-single", action="store_true", help="skip the single-cell drop-in case")
    ap.add_argument("--fp64-batch-steps", type=int, default=100)
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--serving-only", action="store_true", help="print only the serving measurement")
    ap.add_argument("--serve-capacity", type=float, default=0.0,
                    help="with --serving-only: the batch throughput (compartment-steps/s) that sets the "
                         "sustained rate (0: no sustained run)")
    ap.add_argument("--serve-rate", type=float, default=2000.0, help="offered requests/s")
    ap.add_argument("--serve-window", type=float, default=0.5, help="s of arrivals at the offered rate")
    ap.add_argument("--serve-rate-low", type=float, default=10.0, help="a second, low arrival rate")
    ap.add_argument("--serve-window-low", type=float, default=8.0)
    ap.add_argument("--serve-load", type=float, default=0.6,
                    help="sustained run: offered load as a fraction of the batch's capacity")
    ap.add_argument("--serve-window-sustained", type=float, default=6.0)
    ap.add_argument("--serve-chunk", type=int, default=4000)
    ap.add_argument("--serve-admit", type=float, default=0.05, help="s between admission rounds")
    ap.add_argument("--serve-budget", type=float, default=150e9)
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        out = run_reference(args, rank, world)
        if out is not None:
            print(json.dumps(out))
        return 0
    if args.accuracy_full:
        print(json.dumps({"accuracy_full": run_accuracy_full(args)}))
        return 0
    if args.serving_only:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"serving": run_serving(args, args.serve_capacity or None)}))
        return 0
    # the CPU pool is spawned before the first GPU call
    cpu_pool = None
    if rank == 0 and not args.skip_cpu:
        ids = list(range(0, args.cells, max(1, args.cells // args.cpu_cells)))[: args.cpu_cells]
        cpu_pool = CpuPool(ids, args.cells, os.cpu_count() or 1, (2 * args.cpu_chunk + 2) * DT)
    args.config2_pool = None
    if rank == 0 and not args.skip_cpu and not args.skip_config2:
        args.config2_pool = CpuPool(list(range(256)), 256, os.cpu_count() or 1,
                                    (args.config2_cpu_steps + 2) * DT, config=2)
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    out = run_ours(args, rank, world, cpu_pool)
    if cpu_pool is not None:
        cpu_pool.close()
    if args.config2_pool is not None:
        args.config2_pool.close()
    if out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
