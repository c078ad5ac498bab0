"""Whole cells stepped by the oracle in parallel processes, for the GPU parity
tests at workload sizes.  TEST INFRASTRUCTURE: the oracle is the checker.

Processes are started with ``spawn`` (a pool forked after CUDA started in
the parent would hang).  A job names a cell builder of this module and its
arguments, so that each process builds its own cell from the same seeds as
the test does and nothing large is pickled.
"""
import multiprocessing as mp
import os

import numpy as np

DT = 25e-6


def workload_cell(config, seed, i, t_end, n_cells=None):
    """Cell i of a seeded workload (moose_gb300.models.make_cell)."""
    from moose_gb300 import models
    return models.make_cell(config, seed, i, n_cells=n_cells, t_end=t_end)


def cable_cell(n_compt, seed, t_end, n_syn=200, inject=0.5e-9):
    """An unbranched cable of n_compt compartments (soma + n_compt-1 segments of
    10 um x 2 um) with the workload's channels (HH Na/K, Ca(HVA), K(Ca)
    HHChannel2D, CaConc on every compartment), n_syn dual-exponential
    SynChans driven by 5 Hz Poisson trains and a somatic step current."""
    from moose_gb300 import models
    rng = np.random.default_rng([seed, n_compt])
    parent, d, L = models.cable_morphology(n_compt - 1)
    return models.active_cell(parent, d, L, inject=inject, n_syn=n_syn, syn_rate=5.0, rng=rng, t_end=t_end)


BUILDERS = {"workload": workload_cell, "cable": cable_cell}


def _run(job):
    from oracle import OracleCell
    kind, args, nsteps, stride, full_every = job
    m = BUILDERS[kind](*args)
    o = OracleCell(m, DT)
    o.reinit(DT)
    soma = [o.vm()[0]]
    full = []
    for s in range(nsteps // stride):
        o.step(stride)
        soma.append(o.vm()[0])
        if full_every and ((s + 1) * stride) % full_every == 0:
            full.append(o.vm())
    _, t = o.spikes()
    return {"soma": np.array(soma), "full": np.array(full), "vm": o.vm(), "ca": o.ca(), "spikes": np.sort(t)}


def run(jobs, workers=None):
    """Each job = (builder, args, nsteps, stride, full_every): the soma Vm
    every `stride` steps (sample 0 at reinit), every compartment's Vm every
    `full_every` steps (0: never), the final Vm and Ca, the spike times."""
    workers = min(len(jobs), workers or os.cpu_count() or 1)
    with mp.get_context("spawn").Pool(workers) as pool:
        return pool.map(_run, jobs, chunksize=1)
