"""The MOOSE-side binding (moose-core_gb300/cpp/moose_hsolve_bridge.cpp,
linked into the reference build by oracle/build_ref.py) against the
reference's own HSolve.

For each golden model, the reference's pymoose builds the cell and an HSolve
takes it over (HSolve::setup, as a MOOSE script does).  The binding's
fillCellDesc reads that solver's setup vectors and turns them into an
HsCellDesc; the oracle (the CPU restatement, pinned bit-exact to the same
reference build) is created from that description alone, driven the way
the golden script drove the reference (inject changes between runs,
messages into the solver each step, synaptic events at run time) through
the solver's own index space (Hines order), and must reproduce the golden
traces bit for bit -- within 1e-9 where the golden itself is held to that.
The description's indices are mapped back to the script's objects by path
only to compare.

CPU only; skipped where the reference build (oracle/_ref) is absent."""
import ctypes as C
import os
import re
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from loader import load_model, push_pre_reinit, replay_events, replay_messages

REF = os.path.join(ROOT, "oracle", "_ref")
if not os.path.isdir(os.path.join(REF, "moose")):
    pytest.skip("reference build (oracle/_ref) not present", allow_module_level=True)
sys.path.insert(0, REF)
try:
    import moose  # noqa: E402  (the reference's pymoose)
    moose._moose
except (ImportError, AttributeError):
    # the compiled extension is built for the machine that built it only
    pytest.skip("reference build (oracle/_ref) not importable on this machine", allow_module_level=True)
import make_golden_active as mga  # noqa: E402
from moose_gb300.abi import FIELDS, HS_KIND_COMPT, HsCellDesc  # noqa: E402
from oracle import OracleCell, lib  # noqa: E402

_L = C.CDLL(moose._moose.__file__)
_L.hsb_fill_cell_desc.restype = C.POINTER(HsCellDesc)
_L.hsb_fill_cell_desc.argtypes = [C.c_char_p, C.POINTER(C.c_uint32)]
_L.hsb_last_error.restype = C.c_char_p
_L.hsb_free_cell_desc.argtypes = [C.POINTER(HsCellDesc)]
_L.hsb_object_path.argtypes = [C.POINTER(HsCellDesc), C.c_int, C.c_uint32, C.c_char_p, C.c_uint32]


def _paths(d, kind, n):
    buf = C.create_string_buffer(512)
    out = []
    for i in range(n):
        assert _L.hsb_object_path(d, kind, i, buf, 512) >= 0
        out.append(buf.value.decode())
    return out


def _index(paths, pattern):
    """Model index of each solver index, from the object names the golden
    script gave (c<k>, chan<k>, ca<k>, syn<k>, sg<k>)."""
    return np.array([int(re.search(pattern, p).group(1)) for p in paths])


class BridgedCell:
    """The oracle created from the binding's description of the reference
    HSolve, seen through the golden model's indices."""

    def __init__(self, m, dt, dt_setup, ca_advance=1):
        mga.build_moose(m, dt)
        for t in range(8):
            moose.setClock(t, dt)
        h = moose.HSolve("/cell/hsolve")
        h.dt = dt_setup
        h.caAdvance = ca_advance
        h.target = "/cell/c%d" % m.seed
        seed = C.c_uint32()
        d = _L.hsb_fill_cell_desc(b"/cell/hsolve", C.byref(seed))
        assert d, _L.hsb_last_error()
        self._d = d
        self.desc = d.contents
        N = self.desc.n_compt
        assert N == m.n_compt
        # solver index -> model index, per kind, from the objects' names
        self.compt = _index(_paths(d, 0, N), r"/c(\d+)$")
        self.chan = _index(_paths(d, 1, self.desc.n_chan), r"/chan(\d+)$")
        self.pool = _index(_paths(d, 2, self.desc.n_pool), r"/ca(\d+)$")
        self.syn = _index(_paths(d, 4, self.desc.n_syn), r"/syn(\d+)$")
        self.hines = np.empty(N, np.int64)
        self.hines[self.compt] = np.arange(N)
        self.chan_of = {int(k): i for i, k in enumerate(self.chan)}
        self.pool_of = {int(p): i for i, p in enumerate(self.pool)}
        self.syn_of = {int(k): i for i, k in enumerate(self.syn)}
        self.m = m
        oc = OracleCell.__new__(OracleCell)
        oc.model = type("M", (), {"n_compt": N, "pool_compt": np.zeros(self.desc.n_pool)})()
        oc._desc = self.desc
        err = C.create_string_buffer(256)
        oc.h = lib().orc_create(d, seed.value, dt_setup, err, 256)
        assert oc.h, err.value
        self.oc = oc
        oc.set_ca_advance(ca_advance)
        self.step_no = 0
        self.stim = sorted(zip(m.stim_step.tolist(), m.stim_compt.tolist(), m.stim_value.tolist()))

    def close(self):
        # the oracle reads the description while it lives: destroy it first
        if getattr(self, "oc", None) is not None:
            lib().orc_destroy(self.oc.h)
            self.oc.h = None
            self.oc = None
        if getattr(self, "_d", None):
            _L.hsb_free_cell_desc(self._d)
            self._d = None

    def __del__(self):
        self.close()

    # the golden model's description carries things the solver does not
    # hold: the stimulus schedule (a script's inject writes between runs) and
    # the events queued after reinit (Synapse::addSpike)
    def reinit(self, dt):
        self.oc.reinit(dt)
        self.step_no = 0
        m = self.m
        if len(m.ev_syn):
            self.push_events(m.ev_syn, m.ev_time, m.ev_weight)

    def step(self, n):
        end = self.step_no + n
        while self.step_no < end:
            for s, c, v in self.stim:
                if s == self.step_no:
                    self.oc.set(HS_KIND_COMPT, FIELDS["inject"], int(self.hines[c]), v)
            nxt = min([s for s, _, _ in self.stim if s > self.step_no] + [end])
            self.oc.step(nxt - self.step_no)
            self.step_no = nxt

    def vm(self):
        return self.oc.vm()[self.hines]

    def ca(self):
        ca = self.oc.ca()
        out = np.empty(len(ca))
        out[self.pool] = ca
        return out

    def spikes(self):
        return self.oc.spikes()

    def add_inject(self, compt, value):
        self.oc.add_inject(int(self.hines[compt]), value)

    def add_conc(self, chan, conc):
        self.oc.add_conc(self.chan_of[int(chan)], conc)

    def add_ica(self, pool, ica):
        self.oc.add_ica(self.pool_of[int(pool)], ica)

    def push_events(self, syn, time, weight):
        self.oc.push_events([self.syn_of[int(k)] for k in np.atleast_1d(syn)], time, weight)


def _golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    m = load_model(z)
    dt = float(z["dt"])
    dts = float(z["dt_setup"]) if "dt_setup" in z.files else dt
    return z, m, dt, dts


@pytest.mark.parametrize("name", ["active_hh_cable", "active_branched_kca", "active_branched_caadv0"])
def test_bridged_description_reproduces_reference_traces(name):
    z, m, dt, dts = _golden(name)
    c = BridgedCell(m, dt, dts, int(z["ca_advance"]) if "ca_advance" in z.files else 1)
    # the description's own walk numbers the compartments as the solver did
    assert np.array_equal(np.sort(c.compt), np.arange(m.n_compt))
    assert c.desc.n_chan == len(m.chan_compt) and c.desc.n_pool == len(m.pool_compt)
    assert c.desc.n_chan2d == len(m.c2d_compt) and c.desc.n_syn == len(m.syn_compt)
    c.reinit(dt)
    rec = z["rec"]
    stride, n = int(z["stride"]), int(z["nsteps"])
    vm, ca = [c.vm()[rec]], [c.ca()[rec]] if len(m.pool_compt) else []
    for _ in range(n // stride):
        c.step(stride)
        vm.append(c.vm()[rec])
        if len(m.pool_compt):
            ca.append(c.ca()[rec])
    vm = np.array(vm).T
    assert np.array_equal(vm, z["vm"])
    assert np.array_equal(c.vm(), z["final_vm"])
    if len(m.pool_compt):
        assert np.array_equal(np.array(ca).T, z["ca"])
    assert np.array_equal(np.sort(c.spikes()[1]), z["spikes"])


def test_bridged_description_fields_match_the_model():
    """Field by field, the description the binding read from the reference
    solver equals the script's model, permuted into the solver's order."""
    z, m, dt, dts = _golden("active_branched_kca")
    c = BridgedCell(m, dt, dts)
    d, N = c.desc, m.n_compt

    def arr(name, n, dtype=np.float64):
        p = getattr(d, name)
        return np.ctypeslib.as_array(p, shape=(n,)).astype(dtype) if n else np.zeros(0, dtype)

    for f in ("Ra", "Rm", "Cm", "Em", "initVm", "inject"):
        assert np.array_equal(arr(f, N), getattr(m, f)[c.compt]), f
    nc = d.n_chan
    for f in ("chan_Gbar", "chan_Ek", "chan_Xpower", "chan_Ypower", "chan_Zpower", "chan_modulation"):
        assert np.array_equal(arr(f, nc), getattr(m, f)[c.chan]), f
    assert np.array_equal(c.compt[arr("chan_compt", nc, np.int64)], m.chan_compt[c.chan])
    tgt = arr("chan_ca_target", nc, np.int64)
    assert np.array_equal(np.where(tgt >= 0, c.pool[np.maximum(tgt, 0)], -1), m.chan_ca_target[c.chan])
    np_ = d.n_pool
    for f in ("pool_CaBasal", "pool_tau", "pool_ceiling", "pool_floor"):
        assert np.array_equal(arr(f, np_), getattr(m, f)[c.pool]), f
    assert np.array_equal(c.compt[arr("pool_compt", np_, np.int64)], m.pool_compt[c.pool])
    nk = d.n_chan2d
    for f in ("c2d_Gbar", "c2d_Ek", "c2d_Xpower"):
        assert np.array_equal(np.sort(arr(f, nk)), np.sort(getattr(m, f))), f
    ns = d.n_syn
    for f in ("syn_Gbar", "syn_Ek", "syn_tau1", "syn_tau2"):
        assert np.array_equal(arr(f, ns), getattr(m, f)[c.syn]), f


def test_bridged_description_message_destinations():
    """addInject, addConc and iCa into the solver each step (active_msgs:
    StimulusTables in the reference), through the description's indices."""
    z, m, dt, dts = _golden("active_msgs")
    c = BridgedCell(m, dt, dts)
    c.reinit(dt)
    vm, ca = replay_messages(z, c, lambda s: s.step(1))
    assert np.array_equal(vm, z["vm"])
    assert np.array_equal(ca, z["ca"])
    assert np.array_equal(c.vm(), z["final_vm"])


def test_bridged_description_runtime_events():
    """Synaptic events pushed between runs (active_events), the pushes before
    reinit dropped as SimpleSynHandler::vReinit drops them."""
    z, m, dt, dts = _golden("active_events")
    c = BridgedCell(m, dt, dts)
    push_pre_reinit(z, c)
    c.reinit(dt)
    vm = replay_events(z, c, lambda s, n: s.step(n))
    assert np.array_equal(vm, z["vm"])
    assert np.array_equal(c.vm(), z["final_vm"])
    assert np.array_equal(np.sort(c.spikes()[1]), z["spikes"])


def test_bridge_refuses_a_path_without_hsolve():
    seed = C.c_uint32()
    assert not _L.hsb_fill_cell_desc(b"/no/such/solver", C.byref(seed))
    assert b"HSolve" in _L.hsb_last_error()


@pytest.mark.parametrize("name", ["rdes_squid_axon", "rdes_current_pulse", "rdes_ball_and_stick",
                                  "rdes_periodic_syn", "rdes_squid_pulse"])
def test_bridged_description_rdesigneur_known_answers(name):
    """The reference's rdesigneur known-answer models (squid axon with Na/K
    on different voltage grids, current pulse, ball and stick, periodic
    synaptic input, squid current pulse), set up by the reference HSolve and
    described by the binding: the soma trace equals the reference's bit for
    bit and passes the test file's own check."""
    from test_oracle_golden import check_rdes_kat
    z, m, dt, dts = _golden(name)
    c = BridgedCell(m, dt, dts)
    c.reinit(dt)
    stride, n = int(z["stride"]), int(z["nsteps"])
    vm = [c.vm()[0]]
    for _ in range(n // stride):
        c.step(stride)
        vm.append(c.vm()[0])
    vm = np.array(vm)
    assert np.array_equal(vm, z["vm"])
    check_rdes_kat(z, vm)
