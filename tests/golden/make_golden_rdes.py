#!/usr/bin/env python3
"""Known-answer tests of the reference's rdesigneur suite as fixtures.

``tests/rdesigneur/test_32_squid_axon_propgn.py`` (41 soma Vm samples of a
201-compartment squid axon), ``tests/rdesigneur/test_20_currentPulse.py``
(mean, std and histogram of a passive soma's Vm under a current pulse) and
``tests/rdesigneur/test_1_minimalModel.py`` (the zombie fields of that soma
right after setup, a doctest) and ``tests/rdesigneur/test_41_ballAndStick.py``
(a soma and a 10-segment dendrite with per-region Na/K densities; its 61
soma samples at 3 decimals) and ``tests/rdesigneur/test_51_periodic_syn_input.py``
(mean and std of a soma driven by a glu SynChan at 50 Hz) and
``tests/rdesigneur/test_30_squid_currentPulse.py`` (an HH squid soma under a
current pulse: the doctest's first and last samples, mean and std), in the
reference source tree, run their
models under HSolve and compare with values written in the test files.  Here the same models are assembled with
the REFERENCE ``moose`` module the way ``rdesigneur.buildModel`` assembles
them (``python/rdesigneur/rdesigneur.py:232-256``): the cell prototype in
/library, channel prototypes from ``rdesigneurProtos.py`` (loaded as a plain
module: the ``rdesigneur`` package itself imports plotting and 3-D viewer
packages that this image does not have), the C++ ``Neuron``'s
``channelDistribution``, a ``Function`` on tick 12 (every 0.1 ms) driving
the soma's ``inject``, a ``Table`` on tick 8 (every 0.1 ms) reading the
soma's Vm, an ``HSolve`` on the soma, elec ticks at 50 us.  The reference
HSolve runs the model one step at a time; the inject the Function leaves
after step k is what the solver uses from step k+1 (tick 12 runs after the
solver's tick 6), which gives the stimulus schedule.  Before anything is
written, the reference's trace is checked against the test file's expected
values (read from the file with ``ast``) with the test's own tolerance.

Saved per test (``rdes_<name>.npz``): the cell as a ``CellModel`` (``model_*``
keys, gate tables included), the schedule inside it, the reference Table's
samples (``vm``), the plot stride in dt steps, and the KAT values.
Prerequisite: the reference build (``python oracle/build_ref.py``).
"""
import ast
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
from build_ref import source_dir  # noqa: E402
REF_TESTS = os.path.join(source_dir(), "tests", "rdesigneur")
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
sys.path.insert(0, os.path.join(REPO, "moose-core_gb300"))

from make_golden_active import save_model  # noqa: E402
from moose_gb300.abi import CellModel  # noqa: E402

ELEC_DT, PLOT_DT, FUNC_DT = 50e-6, 1e-4, 1e-4


def _literal(node):
    """A number, list, tuple, or np.array(<literal>) from an AST node."""
    if isinstance(node, ast.Call) and getattr(node.func, "attr", None) == "array":
        return np.array(_literal(node.args[0]))
    if isinstance(node, ast.Tuple):
        return tuple(_literal(e) for e in node.elts)
    return ast.literal_eval(node)


def test_file_constants(name):
    """Module-level constants of a reference test file (without running it)."""
    tree = ast.parse(open(os.path.join(REF_TESTS, name)).read())
    out = {}
    for node in tree.body:
        if isinstance(node, ast.Assign) and len(node.targets) == 1 and isinstance(node.targets[0], ast.Name):
            try:
                out[node.targets[0].id] = _literal(node.value)
            except (ValueError, TypeError, SyntaxError):
                pass
    return out


def rdesigneur_call(name, func):
    """The literal keyword arguments of the rd.rdesigneur(...) call inside a
    test function (cellProto, chanDistrib, stimList, ...)."""
    tree = ast.parse(open(os.path.join(REF_TESTS, name)).read())
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == func)
    for node in ast.walk(fn):
        if isinstance(node, ast.Call) and getattr(node.func, "attr", None) == "rdesigneur":
            return {k.arg: ast.literal_eval(k.value) for k in node.keywords}
    raise ValueError("no rdesigneur call in %s.%s" % (name, func))


def test_file_function_array(name, func, var):
    """The literal np.array assigned to `var` inside a test function."""
    tree = ast.parse(open(os.path.join(REF_TESTS, name)).read())
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == func)
    for node in ast.walk(fn):
        if isinstance(node, ast.Assign) and any(getattr(t, "id", None) == var for t in node.targets):
            return _literal(node.value)
    raise ValueError("no %s in %s.%s" % (var, name, func))


def doctest_array_ends(name, func):
    """The first and last values of the array a test function's doctest
    prints with numpy's summarising ellipsis."""
    tree = ast.parse(open(os.path.join(REF_TESTS, name)).read())
    doc = next(ast.get_docstring(n) for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == func)
    body = doc[doc.index("array([") + 7:doc.index("])")]
    head, tail = body.split("...")
    num = lambda part: [float(x) for x in part.replace("\n", " ").split(",") if x.strip()]
    return np.array(num(head)), np.array(num(tail))


def allclose_literal(name, func):
    """The literal list given first to np.allclose inside a test function."""
    tree = ast.parse(open(os.path.join(REF_TESTS, name)).read())
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == func)
    for node in ast.walk(fn):
        if isinstance(node, ast.Call) and getattr(node.func, "attr", None) == "allclose" and \
                isinstance(node.args[0], ast.List):
            return np.array(ast.literal_eval(node.args[0]))
    raise ValueError("no np.allclose literal in %s.%s" % (name, func))


def protos():
    spec = importlib.util.spec_from_file_location(
        "rdesigneurProtos", os.path.join(REPO, "oracle", "_ref", "rdesigneur", "rdesigneurProtos.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def assemble(moose, build_cell, chan_protos, chan_distrib, stim_expr):
    """rdesigneur.buildModel for an elec-only model with one soma Vm plot and
    one inject stimulus (none if stim_expr is None)."""
    for p in ("/model", "/library"):
        if moose.exists(p):
            moose.delete(p)
    moose.Neutral("/library")
    cell = build_cell()
    P = protos()
    for fn, name in chan_protos:
        getattr(P, fn)(name)
    model = moose.Neutral("/model")
    moose.copy(cell, model, "elec")                      # installCellFromProtos
    elec = moose.element("/model/elec")
    elec.buildSegmentTree()
    somas = moose.wildcardFind(elec.path + "/#oma#[ISA=CompartmentBase]")
    soma = max(somas, key=lambda c: c.diameter)
    if chan_distrib:                                    # buildChanDistrib
        flat = []
        for entry in chan_distrib:
            flat += list(entry) + [""]
        elec.channelDistribution = flat
    if stim_expr is not None:                           # _buildStims
        moose.Neutral("/model/stims")
        func = moose.Function("/model/stims/stim0")
        func.expr = stim_expr
        func.doEvalAtReinit = 1
        moose.connect(func, "valueOut", soma, "setInject")
    moose.Neutral("/model/graphs")                      # _buildPlots
    tab = moose.Table("/model/graphs/plot0")
    moose.connect(tab, "requestOut", soma, "getVm")
    hsolve = moose.HSolve(elec.path + "/hsolve")        # _configureHSolve
    hsolve.dt = ELEC_DT
    hsolve.target = soma.path
    for t in range(0, 9):                               # _configureClocks
        moose.setClock(t, ELEC_DT)
    moose.setClock(8, PLOT_DT)
    moose.setClock(12, FUNC_DT)
    return elec, soma, tab


def setup_vm(moose, elec):
    """Vm of every compartment right after the solver's setup (V_ before
    reinit)."""
    return {c.path: c.Vm for c in moose.wildcardFind(elec.path + "/#[ISA=CompartmentBase]")}


def doctest_fields(name, func):
    """`field =value` lines of a test function's doctest (moose.showfield)."""
    tree = ast.parse(open(os.path.join(REF_TESTS, name)).read())
    doc = next(ast.get_docstring(n) for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == func)
    out = {}
    for line in doc.splitlines():
        if "=" in line and not line.lstrip().startswith(">>>"):
            k, v = line.split("=", 1)
            try:
                out[k.strip()] = float(v)
            except ValueError:
                pass
    return out


def run_stepwise(moose, soma, tab, nsteps):
    """Reference run, one dt step per call; the inject seen by the solver
    at each step (the value the Function left after the previous one)."""
    moose.reinit()
    injects = [soma.inject]
    for _ in range(nsteps):
        moose.start(ELEC_DT)
        injects.append(soma.inject)
    clock = moose.element("/clock")
    assert abs(clock.currentTime - nsteps * ELEC_DT) < 0.5 * ELEC_DT, clock.currentTime
    return np.array(tab.vector), np.array(injects)


def extract(moose, elec, soma, inject_seq, vm0, events=None):
    """The solver's cell as a CellModel: compartments in depth-first order
    from the soma along `axial` messages (children in message order),
    channels per compartment in `channel` message order, gate tables read
    from the gates, the inject sequence as a stimulus schedule."""
    order, parent = [], []
    stack = [(soma, -1)]
    while stack:
        c, p = stack.pop()
        idx = len(order)
        order.append(c)
        parent.append(p)
        kids = [moose.element(k) for k in c.neighbors["axial"]]
        stack += [(k, idx) for k in reversed(kids)]
    n = len(order)
    f = lambda name: np.array([getattr(c, name) for c in order], dtype=float)
    gates, gate_index = [], {}

    def gate(ch, which):
        # the prototype's gate: a zombified channel's own gate element
        # crashes the reference module when read, and copies share the
        # prototype's tables anyway
        g = moose.element("/library/" + ch.name + "/" + which)
        key = (g.min, g.max, g.divs, np.asarray(g.tableA).tobytes(), np.asarray(g.tableB).tobytes())
        if key not in gate_index:
            gate_index[key] = len(gates)
            gates.append((g.min, g.max, np.array(g.tableA), np.array(g.tableB)))
        return gate_index[key]

    ch_rows, syn_rows = [], []
    for i, c in enumerate(order):
        for e in c.neighbors["channel"]:
            ch = moose.element(e)
            if ch.className == "SynChan":
                syn_rows.append((i, ch.Gbar, ch.Ek, ch.tau1, ch.tau2, ch.modulation))
                continue
            ch_rows.append(dict(compt=i, Gbar=ch.Gbar, Ek=ch.Ek, Xp=ch.Xpower, Yp=ch.Ypower, Zp=ch.Zpower,
                                xg=gate(ch, "gateX") if ch.Xpower > 0 else -1,
                                yg=gate(ch, "gateY") if ch.Ypower > 0 else -1,
                                inst=int(ch.instant), mod=ch.modulation, X=ch.X, Y=ch.Y))
    col = lambda k, dt: np.array([r[k] for r in ch_rows], dtype=dt)
    nch = len(ch_rows)
    steps = [k for k in range(1, len(inject_seq)) if inject_seq[k] != inject_seq[k - 1]]
    m = CellModel(
        parent=np.array(parent, np.int32), Ra=f("Ra"), Rm=f("Rm"), Cm=f("Cm"), Em=f("Em"),
        initVm=f("initVm"), Vm=np.array([vm0[c.path] for c in order]),
        inject=np.where(np.arange(n) == 0, inject_seq[0], 0.0),
        gates=gates, chan_compt=col("compt", np.uint32), chan_Gbar=col("Gbar", float), chan_Ek=col("Ek", float),
        chan_Xpower=col("Xp", float), chan_Ypower=col("Yp", float), chan_Zpower=col("Zp", float),
        chan_xgate=col("xg", np.int32), chan_ygate=col("yg", np.int32), chan_zgate=np.full(nch, -1, np.int32),
        chan_instant=col("inst", np.int32), chan_modulation=col("mod", float),
        chan_use_conc=np.zeros(nch, np.int32), chan_X=col("X", float), chan_Y=col("Y", float),
        chan_Z=np.zeros(nch), chan_ca_target=np.full(nch, -1, np.int32),
        chan_ca_depend=np.full(nch, -1, np.int32),
        stim_compt=np.zeros(len(steps), np.uint32), stim_step=np.array(steps, np.uint32),
        stim_value=np.array([inject_seq[k] for k in steps]), seed=0)
    if syn_rows:
        sc = lambda j, dt: np.array([r[j] for r in syn_rows], dtype=dt)
        m.syn_compt, m.syn_Gbar, m.syn_Ek = sc(0, np.uint32), sc(1, float), sc(2, float)
        m.syn_tau1, m.syn_tau2, m.syn_modulation = sc(3, float), sc(4, float), sc(5, float)
        ev_syn, ev_time, ev_weight = events
        m.ev_syn = np.asarray(ev_syn, np.uint32)
        m.ev_time = np.asarray(ev_time, float)
        m.ev_weight = np.asarray(ev_weight, float)
    return m


def squid_axon(moose, c):
    """test_32's axon prototype: a 10 um soma and 200 cable segments bent
    along a spiral, built with rdesigneurProtos.buildCompt as the test does."""
    P = protos()
    L, seg = c["comptLen"], c["numAxonSegments"]
    axon = moose.Neuron("/library/axon")
    prev = P.buildCompt(axon, "soma", RM=c["RM"], RA=c["RA"], CM=c["CM"], dia=10e-6, x=0, dx=L)
    theta, x, y = 0, L, 0.0
    for i in range(seg):
        dx, dy = L * np.cos(theta), L * np.sin(theta)
        r = np.sqrt(x * x + y * y)
        theta += L / r
        compt = P.buildCompt(axon, "axon" + str(i), RM=c["RM"], RA=c["RA"], CM=c["CM"], x=x, y=y, dx=dx, dy=dy,
                             dia=c["comptDia"])
        moose.connect(prev, "axial", compt, "raxial")
        prev = compt
        x += dx
        y += dy
    return axon


def ball_and_stick(moose, name, soma_dia, soma_len, dend_dia, dend_len, nseg):
    """rdesigneur's ballAndStick cell prototype (rdesigneur.py:505-521): a
    soma and a dendrite of `nseg` equal segments, rdesigneurProtos.buildCompt
    defaults for RM, RA, CM, Em and initVm."""
    P = protos()
    cell = moose.Neuron("/library/" + name)
    prev = P.buildCompt(cell, "soma", dia=soma_dia, dx=soma_len)
    dx = dend_len / nseg
    x = prev.x
    for i in range(nseg):
        compt = P.buildCompt(cell, "dend" + str(i), x=x, dx=dx, dia=dend_dia)
        moose.connect(prev, "axial", compt, "raxial")
        prev = compt
        x += dx
    return cell


def make():
    import moose
    # test_32: squid axon propagation, 0.04 s
    c = test_file_constants("test_32_squid_axon_propgn.py")
    elec, soma, tab = assemble(moose, lambda: squid_axon(moose, c),
                               [("make_HH_Na", "Na"), ("make_HH_K", "K")],
                               [["Na", "#", "Gbar", "1200"], ["K", "#", "Gbar", "360"]],
                               "(t>0.005 && t<0.2) * 2e-11")
    vm0 = setup_vm(moose, elec)
    nsteps = int(round(0.04 / ELEC_DT))
    vm, inj = run_stepwise(moose, soma, tab, nsteps)
    assert np.allclose(vm[::10], c["expected"]), "reference trace does not reproduce test_32"
    m = extract(moose, elec, soma, inj, vm0)
    np.savez_compressed(os.path.join(HERE, "rdes_squid_axon.npz"), dt=ELEC_DT, nsteps=nsteps,
                        stride=int(round(PLOT_DT / ELEC_DT)), vm=vm, kat_samples=c["expected"], kat_every=10,
                        **save_model(m))
    print("squid axon: %d compartments, %d channels, %d samples, stim steps %s" %
          (m.n_compt, len(m.chan_compt), len(vm), list(m.stim_step)))
    # test_20: passive HH soma, current pulse, 0.3 s
    c = test_file_constants("test_20_currentPulse.py")
    P = protos()
    elec, soma, tab = assemble(moose, lambda: P.makePassiveHHsoma(name="cell"), [], [],
                               "(t>0.1 && t<0.2) * 2e-8")
    vm0 = setup_vm(moose, elec)
    nsteps = int(round(0.3 / ELEC_DT))
    vm, inj = run_stepwise(moose, soma, tab, nsteps)
    mean, std, hist, edges = c["expected"]
    h = np.histogram(vm)
    assert np.allclose(vm.mean(), mean) and np.allclose(vm.std(), std), "test_20 mean/std"
    assert np.allclose(h[0], hist) and np.allclose(h[1], edges), "test_20 histogram"
    m = extract(moose, elec, soma, inj, vm0)
    np.savez_compressed(os.path.join(HERE, "rdes_current_pulse.npz"), dt=ELEC_DT, nsteps=nsteps,
                        stride=int(round(PLOT_DT / ELEC_DT)), vm=vm, kat_mean=mean, kat_std=std,
                        kat_hist=hist, kat_edges=edges, **save_model(m))
    print("current pulse: %d compartments, %d samples, stim steps %s" % (m.n_compt, len(vm), list(m.stim_step)))
    # test_41: ball and stick, Na/K densities per region, 0.06 s.  Its own
    # check averages over every Table, the 3-D viewer's included, which
    # cannot be built here; the test file's 61 soma samples (3 decimals,
    # every 1 ms) are checked to their printed precision instead.
    kw = rdesigneur_call("test_41_ballAndStick.py", "test_ball_and_stick")
    proto = kw["cellProto"][0]
    assert proto[0] == "ballAndStick"
    expected41 = test_file_constants("test_41_ballAndStick.py")["expected"]
    elec, soma, tab = assemble(moose, lambda: ball_and_stick(moose, *proto[1:]),
                               [("make_HH_Na", "Na"), ("make_HH_K", "K")], kw["chanDistrib"],
                               kw["stimList"][0][4])
    vm0 = setup_vm(moose, elec)
    nsteps = int(round(0.06 / ELEC_DT))
    vm, inj = run_stepwise(moose, soma, tab, nsteps)
    assert np.allclose(vm[::10], expected41, rtol=0.0, atol=5e-4 + 1e-12), "test_41 soma samples"
    m = extract(moose, elec, soma, inj, vm0)
    np.savez_compressed(os.path.join(HERE, "rdes_ball_and_stick.npz"), dt=ELEC_DT, nsteps=nsteps,
                        stride=int(round(PLOT_DT / ELEC_DT)), vm=vm, kat_samples=expected41, kat_every=10,
                        kat_atol=5e-4, **save_model(m))
    print("ball and stick: %d compartments, %d channels, stim steps %s" %
          (m.n_compt, len(m.chan_compt), list(m.stim_step)))
    # test_51: a glu SynChan on a soma driven at 50 Hz by a periodic
    # RandSpike (rdesigneur._buildSynInputOnCompt with doPeriodic), 0.3 s.
    # The spike times the RandSpike sends to Synapse::addSpike are recorded
    # by a Table on its spikeOut and become the cell's queued events (the
    # synapse's weight, no delay): RandSpike and SimpleSynHandler share
    # tick 1 and the spike reaches the handler in the step it is sent.
    kw = rdesigneur_call("test_51_periodic_syn_input.py", "test_periodic_syninput")
    proto, stim = kw["cellProto"][0], kw["stimList"][0]
    assert proto[0] == "somaProto" and stim[3] == "periodicsyn"

    def soma_proto():
        cell = moose.Neuron("/library/" + proto[1])   # rdesigneur._buildElecSoma
        P.buildCompt(cell, "soma", dia=proto[2], dx=proto[3])
        return cell

    elec, soma, tab = assemble(moose, soma_proto, [(kw["chanProto"][0][0][:-2], kw["chanProto"][0][1])],
                               kw["chanDistrib"], None)
    syn_path = soma.path + "/" + stim[2] + "/sh/synapse[0]"
    rs = P.make_synInput(name="synInput", parent=syn_path)
    rs.doPeriodic = True
    moose.element(syn_path).weight = float(stim[1])
    moose.connect(rs, "spikeOut", syn_path, "addSpike")
    moose.Neutral("/model/stims")
    func = moose.Function("/model/stims/stim0")
    func.expr = stim[4]
    func.doEvalAtReinit = 1
    moose.connect(func, "valueOut", rs, "setRate")
    spk = moose.Table("/model/graphs/spikes")
    moose.connect(rs, "spikeOut", spk, "input")
    vm0 = setup_vm(moose, elec)
    nsteps = int(round(0.3 / ELEC_DT))
    vm, inj = run_stepwise(moose, soma, tab, nsteps)
    mean, std = test_file_function_array("test_51_periodic_syn_input.py", "test_periodic_syninput", "expected")
    assert np.allclose([mean, std], [vm.mean(), vm.std()], rtol=1e-3), "test_51 mean/std"
    times = np.array(spk.vector)
    w = moose.element(syn_path).weight
    m = extract(moose, elec, soma, inj, vm0, events=(np.zeros(len(times)), times, np.full(len(times), w)))
    np.savez_compressed(os.path.join(HERE, "rdes_periodic_syn.npz"), dt=ELEC_DT, nsteps=nsteps,
                        stride=int(round(PLOT_DT / ELEC_DT)), vm=vm, kat_mean=mean, kat_std=std, kat_rtol=1e-3,
                        **save_model(m))
    print("periodic syn: %d SynChan, %d events" % (len(m.syn_compt), len(m.ev_time)))
    # test_30: HH squid soma (Na/K on the passive soma), current pulse,
    # 0.3 s; its doctest prints the Table's first and last three samples to
    # 8 decimals, and the file gives the trace's mean and std.
    kw = rdesigneur_call("test_30_squid_currentPulse.py", "test_current_pulse_squid")
    assert "cellProto" not in kw
    elec, soma, tab = assemble(moose, lambda: P.makePassiveHHsoma(name="cell"),
                               [("make_HH_Na", "Na"), ("make_HH_K", "K")], kw["chanDistrib"],
                               kw["stimList"][0][4])
    vm0 = setup_vm(moose, elec)
    nsteps = int(round(0.3 / ELEC_DT))
    vm, inj = run_stepwise(moose, soma, tab, nsteps)
    head, tail = doctest_array_ends("test_30_squid_currentPulse.py", "test_current_pulse_squid")
    mean_std = allclose_literal("test_30_squid_currentPulse.py", "test_current_pulse_squid")
    assert np.allclose(vm[:len(head)], head, rtol=0.0, atol=5e-9 + 1e-15), "test_30 first samples"
    assert np.allclose(vm[-len(tail):], tail, rtol=0.0, atol=5e-9 + 1e-15), "test_30 last samples"
    assert np.allclose(mean_std, [vm.mean(), vm.std()]), "test_30 mean/std"
    m = extract(moose, elec, soma, inj, vm0)
    np.savez_compressed(os.path.join(HERE, "rdes_squid_pulse.npz"), dt=ELEC_DT, nsteps=nsteps,
                        stride=int(round(PLOT_DT / ELEC_DT)), vm=vm, kat_head=head, kat_tail=tail,
                        kat_mean=mean_std[0], kat_std=mean_std[1], **save_model(m))
    print("squid pulse: %d compartments, %d channels, stim steps %s" %
          (m.n_compt, len(m.chan_compt), list(m.stim_step)))
    # test_1: the passive soma's zombie fields right after setup (the
    # doctest of test_simple prints them with moose.showfield)
    kat = doctest_fields("test_1_minimalModel.py", "test_simple")
    names = ["Cm", "Em", "Im", "Ra", "Rm", "Vm", "initVm", "inject"]
    elec, soma, tab = assemble(moose, lambda: P.makePassiveHHsoma(name="cell"), [], [], None)
    vm0 = setup_vm(moose, elec)
    for k in names:
        assert np.isclose(getattr(soma, k), kat[k], rtol=1e-12, atol=0.0), (k, getattr(soma, k), kat[k])
    m = extract(moose, elec, soma, [soma.inject], vm0)
    np.savez_compressed(os.path.join(HERE, "rdes_minimal.npz"), dt=ELEC_DT, kat_fields=np.array(names),
                        kat_values=np.array([kat[k] for k in names]),
                        ref_values=np.array([getattr(soma, k) for k in names]), **save_model(m))
    print("minimal model: fields %s" % ", ".join("%s=%r" % (k, kat[k]) for k in names))


if __name__ == "__main__":
    make()
