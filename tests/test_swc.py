"""SWC loading (moose_gb300.swc) against what the reference's ReadSwc builds.

tests/golden/swc/*.swc are seeded synthetic morphologies; swc_golden.npz
holds, for each, the reference loadModel's ReadSwc summary, every
compartment it made (creation order: name, parent, children in message
order, Ra, Rm, Cm, diameter, length, Em, initVm, coordinates) and an
HSolve run of the passive cell with a soma inject (written by
tests/golden/make_golden_swc.py).  The bar is bit-for-bit equality: of the
structure and passive values, and of the oracle's Vm on the loaded cell
with the reference HSolve's.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from moose_gb300 import swc
from oracle import OracleCell

Z = np.load(os.path.join(GOLDEN, "swc_golden.npz"))
FILES = sorted({k.split("/")[0] for k in Z.files if "/" in k})
VALID = [f for f in FILES if not f.startswith("invalid")]
INVALID = [f for f in FILES if f.startswith("invalid")]


def path(name):
    return os.path.join(GOLDEN, "swc", name + ".swc")


@pytest.mark.parametrize("name", FILES)
def test_reader_summary_matches_reference(name):
    s = swc.read_swc(path(name))
    nseg, bad, valid, nbranch = Z[name + "/summary"]
    assert (len(s.segs), s.bad, int(s.valid), len(s.branches)) == (nseg, bad, valid, nbranch)


@pytest.mark.parametrize("name", VALID)
def test_compartments_bit_exact(name):
    c = swc.build(swc.read_swc(path(name)))
    assert c.names == list(Z[name + "/names"])
    assert np.array_equal(c.parent, Z[name + "/parent"])
    kids = [[] for _ in range(len(c))]
    for i, p in enumerate(c.parent):
        if p >= 0:
            kids[p].append(c.names[i])
    assert [",".join(k) for k in kids] == list(Z[name + "/children"])
    for f in ("Ra", "Rm", "Cm", "diameter", "length", "x0", "y0", "z0", "x", "y", "z"):
        assert np.array_equal(getattr(c, f), Z[name + "/" + f]), f
    m = swc.load_swc(path(name))
    assert np.array_equal(m.Em, Z[name + "/Em"]) and np.array_equal(m.initVm, Z[name + "/initVm"])


@pytest.mark.parametrize("name", VALID)
def test_oracle_on_loaded_cell_matches_reference_hsolve(name):
    m = swc.load_swc(path(name))
    m.inject[0] = float(Z["inject"])
    dt, stride, n = float(Z["dt"]), int(Z["stride"]), int(Z["nsteps"])
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    rec = [0, m.n_compt - 1]
    tr = [oc.vm()[rec]]
    for _ in range(n // stride):
        oc.step(stride)
        tr.append(oc.vm()[rec])
    assert np.array_equal(np.array(tr).T, Z[name + "/trace"])
    assert np.array_equal(oc.vm(), Z[name + "/final_vm"])


@pytest.mark.parametrize("name", INVALID)
def test_invalid_files_build_nothing(name):
    s = swc.read_swc(path(name))
    assert not s.valid and len(swc.build(s)) == 0 and len(Z[name + "/names"]) == 0
    with pytest.raises(ValueError):
        swc.load_swc(path(name))


def test_soma_with_one_child_is_rejected(tmp_path):
    # the soma is then inside a branch, not a branch end: the reference makes
    # no compartment for it and cannot attach its child
    p = tmp_path / "one.swc"
    p.write_text("1 1 0 0 0 5 -1\n2 3 10 0 0 1 1\n3 3 20 0 0 1 2\n")
    with pytest.raises(ValueError):
        swc.load_swc(str(p))


def test_atoi_atof_prefixes():
    assert swc._atoi("12abc") == 12 and swc._atoi("  -3") == -3 and swc._atoi("x") == 0
    assert swc._atoi("3.9") == 3
    assert swc._atof("1.5e2x") == 150.0 and swc._atof(".5") == 0.5 and swc._atof("abc") == 0.0
