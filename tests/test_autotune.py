"""Autotuner: the search and the cache on the CPU (a synthetic cost), and on
the GPU a tuned batch that computes exactly what the untuned one does."""
import json

import numpy as np
import pytest

from moose_gb300 import autotune


def test_coordinate_descent_finds_the_best_along_each_knob():
    space = {"packing": [(1, 0), (1, 4096), (2, 0)], "threads_per_cta": [1024, 512, 256],
             "steps_per_launch": [100, 50, 200]}
    cost = {(1, 0): 3.0, (1, 4096): 2.0, (2, 0): 2.5}
    tpc = {1024: 1.0, 512: 0.5, 256: 0.9}
    spl = {100: 0.2, 50: 0.3, 200: 0.1}
    calls = []

    def measure(c):
        calls.append(dict(c))
        return cost[c["packing"]] + tpc[c["threads_per_cta"]] + spl[c["steps_per_launch"]]
    start = {"packing": (1, 0), "threads_per_cta": 1024, "steps_per_launch": 100}
    best, trials = autotune.coordinate_descent(space, measure, start)
    assert best == {"packing": (1, 4096), "threads_per_cta": 512, "steps_per_launch": 200}
    # sum, not product, of the candidate lists (no elim_warps list here)
    assert len(trials) == 1 + 2 + 2 + 2 == len(calls)


def test_packing_may_carry_its_own_eliminator_count():
    space = {"packing": [(1, 0), (1, 8, 8)], "threads_per_cta": [1024], "elim_warps": [4, 8],
             "steps_per_launch": [100]}
    # merged forests are slow with 4 eliminators and fast with 8: trying the
    # packing with its own count finds the pair one knob at a time cannot
    cost = {((1, 0), 4): 0.464, ((1, 0), 8): 0.507, ((1, 8, 8), 4): 0.635, ((1, 8, 8), 8): 0.442}

    def measure(c):
        return cost[(c["packing"], c["elim_warps"])]
    start = {"packing": (1, 0), "threads_per_cta": 1024, "elim_warps": 4, "steps_per_launch": 100}
    best, _ = autotune.coordinate_descent(space, measure, start)
    assert best["packing"] == (1, 8, 8) and best["elim_warps"] == 8


def test_signature_and_cache(tmp_path):
    class M:
        def __init__(self, n, s):
            self.n_compt = n
            self.chan_compt = np.zeros(3 * n)
            self.syn_compt = np.zeros(s)
    a = [M(100, 5), M(2000, 0)]
    b = [M(100, 5), M(2000, 0)]
    c = [M(100, 5), M(2001, 0)]
    assert autotune.signature(a, 1) == autotune.signature(b, 1)
    assert autotune.signature(a, 1) != autotune.signature(c, 1)
    assert autotune.signature(a, 0) != autotune.signature(a, 1)
    path = str(tmp_path / "t.json")
    autotune._save(path, {"k": {"packing": [1, 0], "threads_per_cta": 512}})
    assert json.load(open(path))["k"]["threads_per_cta"] == 512
    assert autotune._load(str(tmp_path / "missing.json")) == {}


@pytest.mark.gpu
def test_tuned_batch_computes_the_same(tmp_path):
    from moose_gb300 import models
    from moose_gb300.abi import HS_PREC_MIXED
    from moose_gb300.batch import Batch
    dt = 25e-6
    kca = models.kca_2d_tables(vdivs=300, cadivs=300)
    cells = []
    for i in range(12):
        rng = np.random.default_rng([21, i])
        parent, d, L = models.branched_morphology(rng, int(rng.integers(30, 300)), 0.5, 4)
        cells.append(models.active_cell(parent, d, L, inject=0.6e-9, n_syn=20, rng=rng, t_end=0.05,
                                        kca_tables=kca, syn_rate=50.0))
    ref = Batch(cells, dt, HS_PREC_MIXED)
    ref.reinit(dt)
    ref.process(300)
    b = Batch(cells, dt, HS_PREC_MIXED)
    space = {"packing": [(1, 0), (1, 256)], "threads_per_cta": [1024, 256], "elim_warps": [4, 2],
             "steps_per_launch": [100, 30]}
    got = autotune.autotune(b, dt, steps=60, warmup=10, space=space, cache=str(tmp_path / "c.json"))
    assert got["threads_per_cta"] in (1024, 256) and got["cached"] is False
    again = autotune.autotune(b, dt, space=space, cache=str(tmp_path / "c.json"))
    assert again["cached"] is True
    b.process(300)
    for i in range(len(cells)):
        assert np.array_equal(b.vm(i), ref.vm(i))
