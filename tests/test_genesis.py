"""GENESIS .p loading (moose_gb300.genesis) against what the reference's
ReadCell builds.

tests/golden/genesis/*.p are seeded synthetic cell files; genesis_golden.npz
holds, for each, every compartment the reference loadModel made (creation
order), every channel's Gbar and Ek, every SynChan's Gbar, Ek and time
constants, CaConc B after zombification, SpikeGen thresholds and an HSolve
run with a soma inject and queued synaptic events (written by
tests/golden/make_golden_genesis.py, which also defines the channel library
used here).  The bar is bit-for-bit equality.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN
from moose_gb300 import genesis
from oracle import OracleCell

sys.path.insert(0, GOLDEN)
from make_golden_genesis import library  # noqa: E402

Z = np.load(os.path.join(GOLDEN, "genesis_golden.npz"))
FILES = sorted({k.split("/")[0] for k in Z.files if "/" in k})
LIB = library(Z)


def path(name):
    return os.path.join(GOLDEN, "genesis", name + ".p")


def with_events(m, name):
    """The synaptic events the reference run queued (after reinit)."""
    if name + "/ev_syn" in Z.files:
        m.ev_syn, m.ev_time, m.ev_weight = Z[name + "/ev_syn"], Z[name + "/ev_time"], Z[name + "/ev_weight"]
    return m


@pytest.mark.parametrize("name", FILES)
def test_compartments_bit_exact(name):
    m = genesis.load_p(path(name), LIB)
    assert m.meta["names"] == list(Z[name + "/names"])
    assert m.meta["classes"] == list(Z[name + "/classes"])
    assert np.array_equal(m.parent, Z[name + "/parent"])
    for f in ("Ra", "Rm", "Cm", "Em", "initVm"):
        assert np.array_equal(getattr(m, f), Z[name + "/" + f]), f
    assert np.array_equal(m.meta["diameter"], Z[name + "/diameter"])
    assert np.array_equal(m.meta["length"], Z[name + "/length"])
    for k, f in enumerate(("x0", "y0", "z0", "x", "y", "z")):
        assert np.array_equal(m.meta["coords"][:, k], Z[name + "/" + f]), f


@pytest.mark.parametrize("name", FILES)
def test_channels_pools_spikegens(name):
    rc = genesis.read_cell(path(name), LIB)
    got = [(i, o[0], o[2]["Gbar"], o[1].Ek) for i, c in enumerate(rc.compts) for o in c.objs
           if isinstance(o[1], (genesis.HHChannelProto, genesis.HHChannel2DProto))]
    assert [g[0] for g in got] == list(Z[name + "/chan_compt"])
    assert [g[1] for g in got] == list(Z[name + "/chan_name"])
    assert np.array_equal([g[2] for g in got], Z[name + "/chan_Gbar"])
    assert np.array_equal([g[3] for g in got], Z[name + "/chan_Ek"])
    m = genesis.load_p(path(name), LIB)
    assert np.array_equal(m.pool_B, Z[name + "/pool_B"])
    assert np.array_equal(m.sg_threshold, Z[name + "/sg_threshold"])
    assert np.array_equal(m.syn_compt, Z[name + "/syn_compt"])
    for f in ("Gbar", "Ek", "tau1", "tau2"):
        assert np.array_equal(getattr(m, "syn_" + f), Z[name + "/syn_" + f]), f


@pytest.mark.parametrize("name", FILES)
def test_oracle_on_loaded_cell_matches_reference_hsolve(name):
    m = with_events(genesis.load_p(path(name), LIB), name)
    m.inject[0] = float(Z["inject"])
    dt, stride, n = float(Z["dt"]), int(Z["stride"]), int(Z["nsteps"])
    rec = Z[name + "/rec"]
    oc = OracleCell(m, dt)
    oc.reinit(dt)
    npool = min(3, len(m.pool_compt))
    vm, ca = [oc.vm()[rec]], [oc.ca()[:npool]]
    for _ in range(n // stride):
        oc.step(stride)
        vm.append(oc.vm()[rec])
        ca.append(oc.ca()[:npool])
    assert np.array_equal(np.array(vm).T, Z[name + "/vm"])
    if npool:
        assert np.array_equal(np.array(ca).T, Z[name + "/ca"])
    assert np.array_equal(oc.spikes()[1], Z[name + "/spikes"])
    assert np.array_equal(oc.vm(), Z[name + "/final_vm"])


def test_unsupported_forms_are_rejected(tmp_path):
    for body in ("*start_cell /other/cell\nsoma none 10 0 0 10\n",
                 # a Compartment prototype under *symmetric
                 "*symmetric\n*compt /library[0]/protoDend\nsoma none 10 0 0 10\n",
                 # a line channel of the same name as a prototype child
                 "*compt /library[0]/protoDend\nsoma none 10 0 0 10 K 300\n",
                 # a SymCompartment on a Compartment: no distal -> proximal message
                 "soma none 10 0 0 10\n*symmetric\nd1 soma 10 0 0 2\n"):
        p = tmp_path / "x.p"
        p.write_text(body)
        with pytest.raises(ValueError):
            genesis.load_p(str(p), LIB)


def test_symmetric_cable_solves_as_the_asymmetric_one():
    """HSolve reads a SymCompartment as a Compartment: the unbranched
    symmetric cable is the asymmetric cable's model, array for array."""
    text = open(path("symmetric_cable")).read()
    sym = genesis.ReadCell(LIB).read(text)
    asym = genesis.ReadCell(LIB).read(text.replace("*symmetric", "*asymmetric"))
    assert all(c.sym for c in sym.compts) and not any(c.sym for c in asym.compts)
    a = genesis.load_p(path("symmetric_cable"), LIB)
    import tempfile
    with tempfile.NamedTemporaryFile("w", suffix=".p", delete=False) as f:
        f.write(text.replace("*symmetric", "*asymmetric"))
    b = genesis.load_p(f.name, LIB)
    os.unlink(f.name)
    for k in ("parent", "Ra", "Rm", "Cm", "Em", "initVm", "chan_compt", "chan_Gbar", "pool_B"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k


def test_symmetric_branch_has_the_sibling_messages_of_readcell(tmp_path):
    """ReadCell joins a symmetric child to everything its parent's
    distalOut reaches -- earlier children and the parent's own siblings --
    by sibling messages, which the reference's tree walk follows without
    end; the model keeps the links and refuses to be described."""
    p = tmp_path / "b.p"
    p.write_text("*symmetric\nsoma none 20 0 0 20\nd1 soma 10 0 0 2\nd2 d1 10 0 0 2\n"
                 "b1 d1 0 10 0 1.5\nb2 b1 0 10 0 1.5\nd3 d2 10 0 0 2\n")
    m = genesis.load_p(str(p), LIB)
    # b1 joins its brother d2; b2 joins its uncle d2; d3 joins what d2's
    # distalOut reaches by then: its brother b1 and b1's child b2
    assert sorted(m.meta["sibling_links"]) == [(3, 2), (4, 2), (5, 3), (5, 4)]
    with pytest.raises(ValueError, match="sibling"):
        m.desc()


def test_comment_block_line_starting_with_star_is_a_command(tmp_path):
    # inside /* */ a line that starts with '*' is still read as a command
    # (ReadCell::innerRead), so *polar below takes effect
    p = tmp_path / "c.p"
    p.write_text("/* block\n*polar\n*/\nsoma none 10 90 90 10\n")
    rc = genesis.read_cell(str(p), LIB)
    assert rc.polar == 1
    assert abs(rc.compts[0].y - 10e-6) < 1e-12


def test_compartment_prototype_path_and_copies(tmp_path):
    """``*compt`` takes a prototype only by its Id::path (``/library[0]/NAME``);
    any other spelling warns and keeps the previous prototype.  A copy
    carries the prototype's children (absolute Gbar), their messages and
    its inject; the line's channels follow them and wire to them."""
    assert genesis.proto_path("protoDend") == "/library[0]/protoDend"
    assert genesis.proto_path("/a/b/c") == "/a[0]/b[0]/c"
    p = tmp_path / "c.p"
    p.write_text("*compt /library/protoSoma\nsoma none 10 0 0 10\n"
                 "*compt /library[0]/protoDend\nd1 soma 10 0 0 2 KCa 20\n"
                 "*compt protoSoma\nd2 d1 10 0 0 2\n")
    rc = genesis.read_cell(str(p), LIB)
    assert sum("bad path" in w for w in rc.warnings) == 2
    soma, d1, d2 = rc.compts
    assert soma.objs == [] and soma.inject == 0.0
    assert [o[0] for o in d1.objs] == ["CaHVA", "Ca_conc", "K", "KCa"]
    assert [o[0] for o in d2.objs] == ["CaHVA", "Ca_conc", "K"]
    assert d1.inject == d2.inject == LIB["protoDend"].inject
    assert d1.objs[0][2]["Gbar"] == LIB["protoDend"].children[0][2]["Gbar"]
    assert d1.objs[0][2]["ca_target"] == "Ca_conc" and d1.objs[3][2]["conc1"] == "Ca_conc"
    # the copies' dictionaries are their own
    d1.objs[2][2]["Gbar"] = 0.0
    assert d2.objs[2][2]["Gbar"] == LIB["protoDend"].children[2][2]["Gbar"]
