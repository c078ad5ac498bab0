"""The elimination plan's cable runs (CellPlan::fRun/bRun, csrc/hs_plan.cpp)
on the host, through tests/cpp/plan_runs_shim.cpp compiled here with g++:
walking the runs the way the FP64 kernels do (pivot carried from row to
row, indices computed) gives M, VMid and V bit-identical to the general
level programs; the single cell's cable is all runs; branched cells keep
their general levels."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from moose_gb300 import models
from moose_gb300.abi import HsCellDesc

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT = os.path.join(HERE, "cpp", "_build")


@pytest.fixture(scope="module")
def lib():
    os.makedirs(OUT, exist_ok=True)
    csrc = os.path.join(REPO, "moose-core_gb300", "csrc")
    srcs = [os.path.join(HERE, "cpp", "plan_runs_shim.cpp"), os.path.join(csrc, "hs_plan.cpp")]
    deps = srcs + [os.path.join(csrc, "hs_plan.h")]
    so = os.path.join(OUT, "libplan_runs_shim.so")
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(p) for p in deps):
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o", so] + srcs +
                       ["-I", csrc], check=True, capture_output=True, text=True)
    L = C.CDLL(so)
    L.plan_runs_check.argtypes = [C.POINTER(HsCellDesc), C.c_uint32, C.POINTER(C.c_uint32)]
    L.plan_runs_check.restype = C.c_int
    return L


def check(L, m, seed):
    d = m.desc()            # holds pointers into m: keep m alive across the call
    st = (C.c_uint32 * 5)()
    rc = L.plan_runs_check(C.byref(d), seed, st)
    return rc, list(st)


@pytest.mark.parametrize("seed", [0, 100, 200])
def test_single_cell_cable_is_all_runs(lib, seed):
    m = models.config1_cell()
    rc, (n, fr, br, fl, bl) = check(lib, m, seed)
    assert rc == 0
    assert (n, fr, br, fl, bl) == (201, 200, 200, 201, 201)


def test_random_trees_bit_identical(lib):
    rng = np.random.default_rng(5)
    rows = 0
    for _ in range(40):
        n = int(rng.integers(2, 800))
        parent, d, L = models.branched_morphology(rng, n, float(rng.uniform(0.02, 0.9)), int(rng.integers(2, 7)))
        m = models.active_cell(parent, d, L, gkca=0.0)
        rc, st = check(lib, m, int(rng.integers(0, n)))
        assert rc == 0
        rows += st[1] + st[2]
    assert rows > 0


def test_unbranched_tails_on_a_branched_cell(lib):
    """A soma with two long cables and a short branch: runs inside the
    cables, general levels at the junction."""
    parent = [-1] + list(range(0, 60)) + [0] + list(range(61, 120)) + [30, 121, 122]
    n = len(parent)
    d, L = np.full(n, 2e-6), np.full(n, 10e-6)
    m = models.active_cell(np.array(parent, np.int32), d, L, gkca=0.0)
    for seed in (0, 45, n - 1):
        rc, (nn, fr, br, fl, bl) = check(lib, m, seed)
        assert rc == 0 and nn == n
        assert fr > 0 and br > 0 and fr < n - 1


def waves(L, m, seed):
    d = m.desc()
    st = (C.c_uint32 * 4)()
    L.plan_waves_check.argtypes = [C.POINTER(HsCellDesc), C.c_uint32, C.POINTER(C.c_uint32)]
    rc = L.plan_waves_check(C.byref(d), seed, st)
    return rc, list(st)


def test_forward_waves_bit_identical(lib):
    """The forward sweep as waves of fused updates, each wave run last to
    first, gives M, VMid and V bit-identical to the level programs: random
    trees (junctions of rank 1 to 6, seeds anywhere), workload-like cells up
    to 10,000 compartments and a rank-41 star.  Branched cells take waves,
    the cable keeps its runs."""
    rng = np.random.default_rng(8)
    taken = 0
    for _ in range(40):
        n = int(rng.integers(2, 900))
        parent, d, L = models.branched_morphology(rng, n, float(rng.uniform(0.02, 0.9)), int(rng.integers(2, 7)))
        m = models.active_cell(parent, d, L, gkca=0.0)
        rc, st = waves(lib, m, int(rng.integers(0, n)))
        assert rc == 0
        taken += st[1] > 0
    assert taken > 20
    for n in (2000, 10000):
        parent, d, L = models.branched_morphology(np.random.default_rng(n), n, 0.5, 4)
        m = models.active_cell(parent, d, L, gkca=0.0)
        rc, (nn, nw, nf, nl) = waves(lib, m, m.seed)
        assert rc == 0 and nw > 0 and nw < 2 * nl
    star = [-1] + [0] * 40 + list(range(1, 41))
    m = models.active_cell(np.array(star, np.int32), np.full(81, 2e-6), np.full(81, 10e-6), gkca=0.0)
    rc, st = waves(lib, m, 0)
    assert rc == 0 and st[1] > 0
    rc, st = waves(lib, models.config1_cell(), 0)
    assert rc == 0 and st[1] == 0
