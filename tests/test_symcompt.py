"""SymCompartment cells under HSolve (hsolve/HSolve.cpp:505-513,
hsolve/HSolveUtils.cpp:36-53): a branched cell wired with distal ->
proximal, sphere -> proximalOnly and cylinder -> proximalOnly links, set up
by the reference HSolve and described by the MOOSE-side binding
(symcompt_branched.npz, tests/golden/make_golden_symcompt.py).  The oracle
(on the CPU) and the FP64 drop-in (on the GPU), given that description
alone, reproduce the reference's Vm traces, spike times and final Vm bit
for bit.  The GENESIS reader's *symmetric cable is covered with the other
.p files in test_genesis.py / test_gpu_genesis.py."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from loader import load_model
from oracle import OracleCell

Z = np.load(os.path.join(GOLDEN, "symcompt_branched.npz"))


def _run(solver, advance):
    rec, stride, n = Z["rec"], int(Z["stride"]), int(Z["nsteps"])
    vm = [solver.vm()[rec]]
    for _ in range(n // stride):
        advance(stride)
        vm.append(solver.vm()[rec])
    return np.array(vm).T


def _check(vm, final, spikes):
    assert np.array_equal(vm, Z["vm"])
    assert np.array_equal(final[Z["final_index"]], Z["final_vm"])
    assert np.array_equal(spikes, Z["spikes"])
    assert len(spikes) > 0


def test_branched_symcompartment_cell_oracle_bit_exact():
    m = load_model(Z)
    # the tree the reference walked: one root, a branch point, the spines
    assert (m.parent < 0).sum() == 1
    assert np.bincount(m.parent[m.parent >= 0]).max() == 3      # d2: d3 and two spines
    dt = float(Z["dt"])
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    vm = _run(oc, oc.step)
    _check(vm, oc.vm(), oc.spikes()[1])


@pytest.mark.gpu
def test_branched_symcompartment_cell_dropin_bit_exact():
    from moose_gb300.hsolve import HSolve
    m = load_model(Z)
    dt = float(Z["dt"])
    h = HSolve(m, dt=dt)
    h.target = m.seed
    h.reinit(dt)
    vm = _run(h, h.process)
    _check(vm, h.vm(), h.spikes()[1])
    h.close()
