#!/usr/bin/env python3
"""Generate the golden vectors under tests/golden/ from the REFERENCE itself.

Run in a container that has the reference sources and its build
(``python oracle/build_ref.py`` first).  Nothing at test time runs the
reference: the tests read only the files written here.

1. ``passive_kat.json`` -- the reference's own ``HinesMatrix`` and
   ``HSolvePassive`` (linked by ``oracle/ref_passive_harness``) on
   (a) the nine hand-numbered cells of the reference's unit tests
       (``hsolve/HinesMatrix.cpp:478-755``, ``hsolve/HSolvePassive.cpp:452-987``:
       same child lists, Ra = 15+3i, Rm = 45+15i, Cm = 500+200i^2,
       Em = -0.06, V = -0.06+0.01i, dt = 1), and
   (b) seeded random trees with junctions of rank up to 5,
   dumping A, B, the forward-eliminated A/B, VMid and V of two passes as hex
   floats (exact bits).
2. ``active_*.npz`` -- traces of full models stepped by the reference
   ``moose`` Python module with an HSolve (see ``active_models()``).

The other fixtures have their own scripts beside this one, run the same way
after the reference build: ``make_golden_msgs.py`` (message destinations),
``make_golden_events.py`` (synaptic events pushed at run time),
``make_golden_rdes.py`` (the reference's rdesigneur known-answer tests),
``make_golden_swc.py`` and ``make_golden_genesis.py`` (the loaders).
"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(REPO, "oracle", "_ref", "ref_passive_harness")

# The nine cells of the reference's testHinesMatrix/testHSolvePassive, as
# child lists in Hines order.
REFERENCE_CELLS = [
    [[], [0], [1], [], [3], [], [5], [4, 6], [7], [8], [], [10], [], [12], [11, 13],
     [14, 16], [17], [2, 9, 18], [19], []],
    [[], [], [0, 1, 3], []],
    [[2], [], [1, 3], []],
    [[], [], [0, 1], [2]],
    [[], [2], [0, 4], [], [3, 5], []],
    [[], [], [], [4], [0, 1, 2, 5, 6], [], []],
    [[]],
    [[], [0, 2], []],
    [[1], [2], []],
]


def random_tree_hines(rng, n, maxchild):
    """A random tree relabelled into the Hines order of the oracle's walk."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    from oracle import OracleCell
    sys.path.insert(0, os.path.join(REPO, "moose-core_gb300"))
    from moose_gb300.abi import CellModel
    parent = np.full(n, -1, np.int32)
    nchild = np.zeros(n, int)
    for i in range(1, n):
        while True:
            p = int(rng.integers(0, i))
            if nchild[p] < maxchild:
                break
        parent[i] = p
        nchild[p] += 1
    ones = np.ones(n)
    m = CellModel(parent=parent, Ra=ones, Rm=ones, Cm=ones, Em=-0.06 * ones,
                  initVm=-0.06 * ones, Vm=-0.06 * ones, inject=0 * ones, seed=0)
    oc = OracleCell(m, 1.0)
    order = oc.hines_order()                 # hines -> model
    hines_of = np.empty(n, int)
    hines_of[order] = np.arange(n)
    children = [[] for _ in range(n)]
    for i in range(n):                        # axial message order: child index
        if parent[i] >= 0:
            children[hines_of[parent[i]]].append(int(hines_of[i]))
    return children


def passive_params(n):
    i = np.arange(n, dtype=np.float64)
    return dict(Ra=15.0 + 3.0 * i, Rm=45.0 + 15.0 * i, Cm=500.0 + 200.0 * i * i,
                Em=np.full(n, -0.06), V=-0.06 + 0.01 * i)


def run_harness(cells):
    lines = []
    for c in cells:
        n = len(c["children"])
        lines.append("%d %s" % (n, float(c["dt"]).hex()))
        for ch in c["children"]:
            lines.append(" ".join([str(len(ch))] + [str(x) for x in ch]))
        for k in ("Ra", "Rm", "Cm", "Em", "V"):
            lines.append(" ".join(float(x).hex() for x in c[k]))
    out = subprocess.run([HARNESS], input="\n".join(lines) + "\n", capture_output=True,
                         text=True, check=True).stdout
    recs, cur = [], None
    for line in out.splitlines():
        tag, *vals = line.split()
        if tag == "CELL":
            cur = {"passes": []}
            recs.append(cur)
        elif tag == "A0":
            cur["A0"] = vals
        elif tag == "B":
            cur["passes"].append({"B": vals})
        else:
            cur["passes"][-1][tag] = vals
    return recs


def make_passive():
    rng = np.random.default_rng(20240611)
    cells = []
    for k, ch in enumerate(REFERENCE_CELLS):
        d = {"name": "reference_cell_%d" % (k + 1), "children": ch, "dt": 1.0}
        d.update({a: b.tolist() for a, b in passive_params(len(ch)).items()})
        cells.append(d)
    for k, (n, mc) in enumerate([(12, 5), (30, 4), (57, 3), (80, 5), (120, 2), (200, 4)]):
        ch = random_tree_hines(rng, n, mc)
        d = {"name": "random_%d_n%d_maxchild%d" % (k, n, mc), "children": ch,
             "dt": float(rng.choice([1.0, 25e-6, 50e-6]))}
        i = np.arange(n, dtype=np.float64)
        d.update(Ra=(1e6 * (1 + rng.random(n))).tolist(), Rm=(1e9 * (1 + rng.random(n))).tolist(),
                 Cm=(1e-12 * (1 + rng.random(n))).tolist(), Em=(-0.065 + 0.01 * rng.random(n)).tolist(),
                 V=(-0.07 + 0.03 * rng.random(n)).tolist())
        cells.append(d)
    recs = run_harness(cells)
    for c, r in zip(cells, recs):
        # dense matrices -> nonzero triplets [i, j, hex]
        n = len(c["children"])
        for key, holder in [("A0", r)] + [("FA", ps) for ps in r["passes"]]:
            vals = holder[key]
            holder[key] = [[k // n, k % n, v] for k, v in enumerate(vals) if float.fromhex(v) != 0.0]
        c["reference"] = r
        for k in ("Ra", "Rm", "Cm", "Em", "V"):
            c[k] = [float(x).hex() for x in c[k]]
        c["dt"] = float(c["dt"]).hex()
    with open(os.path.join(HERE, "passive_kat.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py",
                   "source": "reference HinesMatrix/HSolvePassive via oracle/ref_passive_harness",
                   "cells": cells}, f, separators=(",", ":"))
    print("wrote passive_kat.json with", len(cells), "cells")


if __name__ == "__main__":
    what = sys.argv[1:] or ["passive", "active"]
    if "passive" in what:
        make_passive()
    if "active" in what:
        from make_golden_active import make_active
        make_active()
