"""Autotuner for the batched HSolve: picks the packing and launch shape.

The knobs (``HsBatchTuning``): threads per CTA, CTAs per SM and forest size
(which set how cells are packed into shared-memory forests), the warps that
eliminate while the others assemble (mixed precision), and dt steps per
launch.  Every choice computes the same results (bit-identical, tested), so
the tuner only measures: for each candidate it (re)packs the batch, reinits
it, runs a few warm-up steps, then times ``steps`` dt steps with CUDA events
on the batch's stream (``Batch.kernel_time``), and keeps the fastest.

Search: coordinate descent from the defaults -- first the packing (CTAs per
SM x forest size, each a re-layout), then threads per CTA, eliminator warps
and steps per launch -- so the number of timed runs grows with the sum, not
the product, of the candidate lists.  Packing and eliminator count interact
(forests of a few compartments merge every cell of a CTA into one forest
whose level sweep wants more eliminator warps), so a packing entry may carry
its own eliminator count as a third element, tried together.  Results are cached per workload signature in a JSON
file so that a repeated workload skips the search.
"""
import hashlib
import json
import os

import numpy as np

from .abi import HS_PREC_FP64

MIXED_SPACE = {
    # (ctas_per_sm, forest_nodes[, elim_warps])
    "packing": [(1, 0), (1, 8, 8), (1, 6000), (1, 4096), (2, 0)],
    "threads_per_cta": [1024, 768, 512],
    "elim_warps": [4, 5, 3, 8],
    "steps_per_launch": [100, 50, 200],
}
FP64_SPACE = {
    "packing": [(4, 0), (2, 0), (8, 0)],
    "threads_per_cta": [256, 128],
    "elim_warps": [0],
    "steps_per_launch": [100, 50, 200],
}


def signature(cells, precision):
    """A key for the workload: cell count, compartment-count histogram,
    channel/synapse counts and precision."""
    n = np.array([m.n_compt for m in cells])
    hist = np.histogram(np.log10(np.maximum(n, 1)), bins=8, range=(0, 5))[0]
    chans = sum(len(m.chan_compt) for m in cells)
    syns = sum(len(m.syn_compt) for m in cells)
    key = "%d|%d|%s|%d|%d|%d" % (precision, len(cells), ",".join(map(str, hist)), int(n.sum()), chans, syns)
    return hashlib.sha1(key.encode()).hexdigest()[:16]


def default_cache():
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "moose_gb300", "autotune.json")


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(path, table):
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def coordinate_descent(space, measure, start):
    """Minimise `measure(config) -> ms per step` over `space`, one knob at a
    time starting from `start`; returns (best config, trials)."""
    best = dict(start)
    best_t = measure(best)
    trials = [(dict(best), best_t)]
    for knob in ("packing", "threads_per_cta", "elim_warps", "steps_per_launch"):
        for v in space.get(knob, ()):
            if best.get(knob) == v:
                continue
            cand = dict(best)
            cand[knob] = v
            if knob == "packing" and len(v) > 2:
                cand["elim_warps"] = v[2]
            t = measure(cand)
            trials.append((dict(cand), t))
            if t < best_t:
                best, best_t = cand, t
    return best, trials


def autotune(batch, dt, steps=200, warmup=50, space=None, cache=None, use_cache=True):
    """Tune `batch` (a ``Batch``) in place and return the chosen tuning as a
    dict: threads_per_cta, ctas_per_sm, forest_nodes, steps_per_launch,
    ms_per_step.  The batch is left re-laid-out for the choice and reinited
    (recording and inject targets of a mixed batch must be registered after
    tuning)."""
    prec = batch.precision
    space = space or (FP64_SPACE if prec == HS_PREC_FP64 else MIXED_SPACE)
    cache = cache or default_cache()
    key = signature(batch.cells, prec)
    table = _load(cache) if use_cache else {}

    def apply(cfg):
        cps, fn = cfg["packing"][:2]
        batch.tune(threads_per_cta=cfg["threads_per_cta"], ctas_per_sm=cps,
                   steps_per_launch=cfg["steps_per_launch"], forest_nodes=fn,
                   elim_warps=cfg.get("elim_warps") or 0)
        batch.reinit(dt)

    def measure(cfg):
        apply(cfg)
        batch.process(warmup)
        batch.sync()
        batch.kernel_time()
        batch.process(steps)
        batch.sync()
        ms, n = batch.kernel_time()
        return ms * n / steps if n else float("inf")

    if key in table:
        hit = table[key]
        cfg = {"packing": tuple(hit["packing"]), "threads_per_cta": hit["threads_per_cta"],
               "elim_warps": hit.get("elim_warps", 0), "steps_per_launch": hit["steps_per_launch"]}
        apply(cfg)
        out = dict(hit)
        out["cached"] = True
        return out
    p0 = tuple(space["packing"][0])
    start = {"packing": p0, "threads_per_cta": space["threads_per_cta"][0],
             "elim_warps": p0[2] if len(p0) > 2 else space.get("elim_warps", [0])[0],
             "steps_per_launch": space["steps_per_launch"][0]}
    best, trials = coordinate_descent(space, measure, start)
    apply(best)
    out = {"packing": list(best["packing"]), "threads_per_cta": best["threads_per_cta"],
           "elim_warps": best["elim_warps"], "steps_per_launch": best["steps_per_launch"],
           "ms_per_step": min(t for _, t in trials), "trials": len(trials)}
    if use_cache:
        table[key] = out
        _save(cache, table)
    out = dict(out)
    out["cached"] = False
    return out
