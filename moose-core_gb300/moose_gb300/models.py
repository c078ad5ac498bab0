"""Seeded synthetic cells for the HSolve workloads, as ``CellModel`` objects.

Rate tables follow the reference prototypes:
  * HH squid Na (m^3 h) and K (n^4): ``python/rdesigneur/rdesigneurProtos.py:65-116``
    (A = alpha, B = alpha + beta, rest offset EREST_ACT_HH = -70 mV), tabulated
    here over vMin = -0.1 V .. vMax = 0.05 V with 3000 divisions.
  * high-voltage Ca (m^2 h, Traub): ``rdesigneurProtos.py:199-245`` (``make_Ca``),
    feeding the compartment's CaConc through IkOut (HSolve's caTarget path).
  * Ca-dependent K as an HHChannel2D on (Vm, Ca) with ``VOLT_C1_INDEX``:
    a BK-type gate after Moczydlowski & Latorre (1983), Ca tabulated over
    0..1 mM with 3000 divisions.
Compartment passive properties follow ``rdesigneurProtos.buildCompt``
(``rdesigneurProtos.py:620-638``): Ra = RA*L/(pi d^2/4), Rm = RM/(pi d L),
Cm = CM*pi d L.  CaConc B follows ``biophysics/CaConcBase.cpp:259-269``.
"""
import math

import numpy as np

from .abi import HS_DEP, CellModel

EREST_ACT = -0.060
EREST_ACT_HH = -0.070
ECA = 0.080
FARADAY = 96485.3365
PI = 3.14159265359

# constants of the reference's CaConcBase::updateDimensions (basecode/header.h)
MOOSE_PI = 3.141592653589793
MOOSE_FARADAY = 96485.3415

VMIN, VMAX, VDIVS = -0.1, 0.05, 3000
CAMIN, CAMAX, CADIVS = 0.0, 1.0, 3000


def _vgrid(vmin=VMIN, vmax=VMAX, vdivs=VDIVS):
    return np.linspace(vmin, vmax, vdivs + 1)


def _vtrap(num, u, scale):
    """num / (exp(u/scale) - 1) with its limit num/(u/scale) -> scale at u = 0."""
    den = np.expm1(u / scale)
    small = np.abs(u) < 1e-9
    safe = np.where(small, 1.0, den)
    return np.where(small, scale, num / safe)


def hh_na_tables(vmin=VMIN, vmax=VMAX, vdivs=VDIVS):
    """(m_A, m_B), (h_A, h_B) of the squid Na channel."""
    v = _vgrid(vmin, vmax, vdivs) - EREST_ACT_HH
    u = 25.0 - v * 1e3
    m_alpha = 1e3 * _vtrap(u, u, 10.0) / 10.0
    m_beta = 1e3 * 4.0 * np.exp(-v * 1e3 / 18.0)
    h_alpha = 1e3 * 0.07 * np.exp(-v / 20e-3)
    h_beta = 1e3 * 1.0 / (np.exp((30e-3 - v) / 10e-3) + 1.0)
    return (m_alpha, m_alpha + m_beta), (h_alpha, h_alpha + h_beta)


def hh_k_tables(vmin=VMIN, vmax=VMAX, vdivs=VDIVS):
    """(n_A, n_B) of the squid K channel."""
    v = _vgrid(vmin, vmax, vdivs) - EREST_ACT_HH
    u = 10.0 - v * 1e3
    n_alpha = 1e3 * _vtrap(u, u, 10.0) / 100.0
    n_beta = 1e3 * 0.125 * np.exp(-v * 1e3 / 80.0)
    return (n_alpha, n_alpha + n_beta)


def ca_hva_tables(vmin=VMIN, vmax=VMAX, vdivs=VDIVS):
    """(x_A, x_B), (y_A, y_B) of the Traub high-voltage Ca channel."""
    v = _vgrid(vmin, vmax, vdivs)
    # alpha = 1.6e3 / (1 + exp((V - 0.005)/-0.01389)) with EREST_ACT = -0.06
    xa = 1.6e3 / (1.0 + np.exp((v + (-1.0 * (0.065 + EREST_ACT))) / -0.01389))
    # beta = (A + B V) / (C + exp((V + D)/F)), A = -20e3 (0.0511 + EREST_ACT),
    # B = 20e3, C = -1, D = -(0.0511 + EREST_ACT), F = 5e-3
    u = v + (-1.0 * (0.0511 + EREST_ACT))
    xb = 20e3 * _vtrap(u, u, 5e-3)
    ya = np.where(v > EREST_ACT, 5.0 * np.exp(-50.0 * (v - EREST_ACT)), 5.0)
    yb = np.full_like(v, 5.0)
    return (xa, xa + xb), (ya, yb)


def kca_2d_tables(vmin=VMIN, vmax=VMAX, vdivs=VDIVS, camin=CAMIN, camax=CAMAX, cadivs=CADIVS):
    """A[v][ca], B[v][ca] of a BK-type Ca- and voltage-dependent K gate."""
    v = _vgrid(vmin, vmax, vdivs)[:, None]
    ca = np.linspace(camin, camax, cadivs + 1)[None, :]
    FoverRT = FARADAY / (8.314 * (273.15 + 35.0))
    abar, bbar = 480.0, 280.0            # 1/s
    k1, k2 = 0.18, 0.011                  # mM
    d1, d2 = 0.84, 1.0
    alpha = abar * ca / (ca + k1 * np.exp(-2.0 * d1 * FoverRT * v))
    beta = bbar / (1.0 + ca / (k2 * np.exp(-2.0 * d2 * FoverRT * v)))
    return alpha, alpha + beta


# ---------------------------------------------------------------------------
# morphology

def cable_morphology(n_cable, soma_dia=20e-6, soma_len=20e-6, dia=2e-6, seg_len=10e-6):
    """Soma (index 0) with an unbranched cable of n_cable segments."""
    n = n_cable + 1
    parent = np.arange(-1, n - 1, dtype=np.int32)
    d = np.full(n, dia)
    L = np.full(n, seg_len)
    d[0], L[0] = soma_dia, soma_len
    return parent, d, L


def branched_morphology(rng, n, branch_p=0.5, max_children=2, soma_dia=20e-6,
                        soma_len=20e-6, dia_median=1.5e-6, dia_sigma=0.4,
                        len_range=(5e-6, 20e-6)):
    """Soma plus a random dendritic tree of n-1 compartments.

    Growth from a random open tip: each tip gets one child, or with
    probability ``branch_p`` a branch point of 2..max_children children.
    """
    parent = np.full(n, -1, np.int32)
    tips = [0]
    count = 1
    while count < n:
        t = tips.pop(int(rng.integers(len(tips))))
        k = 1
        if rng.random() < branch_p:
            k = 2 if max_children <= 2 else int(rng.integers(2, max_children + 1))
        for _ in range(k):
            if count >= n:
                break
            parent[count] = t
            tips.append(count)
            count += 1
    d = np.exp(rng.normal(math.log(dia_median), dia_sigma, n))
    L = rng.uniform(len_range[0], len_range[1], n)
    d[0], L[0] = soma_dia, soma_len
    return parent, d, L


def caconc_B(d, L, thick):
    """B of a CaConc shell as `CaConcBase::updateDimensions` computes it
    (biophysics/CaConcBase.cpp:259-269).  The reference HSolve always ends up
    with this B: zombification writes thick/length/diameter back after B and
    each of those setters recomputes B from the geometry."""
    vol = MOOSE_PI * d * d * L * 0.25
    core = d / 2.0 - thick
    shell = (thick > 0) & (thick < d / 2.0)
    vol = np.where(shell, vol - MOOSE_PI * core * core * L, vol)
    return 1.0 / (2 * MOOSE_FARADAY * vol)


def passive(d, L, RM=1.0, RA=1.0, CM=0.01):
    xa = d * d * PI / 4.0
    sa = L * d * PI
    return L * RA / xa, RM / sa, CM * sa, sa


# ---------------------------------------------------------------------------
# cells

def _hh_channels(n, area, gna=1200.0, gk=360.0, na_gates=(0, 1), k_gate=2):
    """Na then K on every compartment (message order: Na first)."""
    comp = np.repeat(np.arange(n, dtype=np.uint32), 2)
    gbar = np.empty(2 * n)
    gbar[0::2] = gna * area
    gbar[1::2] = gk * area
    ek = np.tile([50e-3, -77e-3], n)
    xp = np.tile([3.0, 4.0], n)
    yp = np.tile([1.0, 0.0], n)
    xg = np.tile([na_gates[0], k_gate], n).astype(np.int32)
    yg = np.tile([na_gates[1], -1], n).astype(np.int32)
    return dict(comp=comp, gbar=gbar, ek=ek, xp=xp, yp=yp, zp=np.zeros(2 * n),
                xg=xg, yg=yg, zg=np.full(2 * n, -1, np.int32),
                tgt=np.full(2 * n, -1, np.int32))


def _steady(A, B, vmin, vmax, v):
    """A/B at v by linear interpolation on the gate grid (initial gate state)."""
    x = np.linspace(vmin, vmax, len(A))
    return np.interp(v, x, A) / np.interp(v, x, B)


def config1_cell(n_cable=200, inject=0.5e-9, t_on=0.05, t_off=0.45, dt=25e-6):
    """Single cell of the 201-compartment HH cable workload.

    Soma 20 um x 20 um plus 200 segments of 10 um x 2 um, RA = 1 ohm m,
    RM = 1 ohm m^2, CM = 0.01 F/m^2, Em = -54.4 mV, HH Na/K everywhere
    (gbar 1200 / 360 S/m^2), step of `inject` into the soma from t_on to t_off.
    """
    parent, d, L = cable_morphology(n_cable)
    Ra, Rm, Cm, area = passive(d, L)
    n = len(parent)
    (mA, mB), (hA, hB) = hh_na_tables()
    nA, nB = hh_k_tables()
    gates = [(VMIN, VMAX, mA, mB), (VMIN, VMAX, hA, hB), (VMIN, VMAX, nA, nB)]
    ch = _hh_channels(n, area)
    v0 = -0.065
    X0 = np.where(ch["xg"] == 0, _steady(mA, mB, VMIN, VMAX, v0), _steady(nA, nB, VMIN, VMAX, v0))
    Y0 = np.where(ch["yg"] == 1, _steady(hA, hB, VMIN, VMAX, v0), 0.0)
    on = int(round(t_on / dt))
    off = int(round(t_off / dt))
    return CellModel(
        parent=parent, Ra=Ra, Rm=Rm, Cm=Cm, Em=np.full(n, -54.4e-3),
        initVm=np.full(n, v0), Vm=np.full(n, v0), inject=np.zeros(n),
        gates=gates,
        chan_compt=ch["comp"], chan_Gbar=ch["gbar"], chan_Ek=ch["ek"],
        chan_Xpower=ch["xp"], chan_Ypower=ch["yp"], chan_Zpower=ch["zp"],
        chan_xgate=ch["xg"], chan_ygate=ch["yg"], chan_zgate=ch["zg"],
        chan_instant=np.zeros(2 * n, np.int32), chan_modulation=np.ones(2 * n),
        chan_use_conc=np.zeros(2 * n, np.int32), chan_X=X0, chan_Y=Y0, chan_Z=np.zeros(2 * n),
        chan_ca_target=ch["tgt"], chan_ca_depend=ch["tgt"].copy(),
        sg_compt=np.array([0], np.uint32), sg_threshold=np.array([0.0]),
        sg_refractT=np.array([1e-3]), sg_edge=np.array([1], np.int32),
        stim_compt=np.array([0, 0], np.uint32), stim_step=np.array([on, off], np.uint32),
        stim_value=np.array([inject, 0.0]), seed=0)


def active_cell(parent, d, L, inject=0.5e-9, n_syn=0, syn_rate=5.0, t_end=1.0,
                rng=None, gca=5.0, gkca=50.0, kca_tables=None, ca_thickness=0.1e-6,
                syn_weight_median=0.5e-9, syn_weight_sigma=0.5, cadivs=CADIVS,
                inject_step=0, passive_props=None):
    """HH Na/K + Ca(HVA) + K(Ca) HHChannel2D + CaConc on every compartment.

    The Ca channel feeds the compartment's CaConc (IkOut -> current, HSolve's
    caTarget) and the CaConc feeds the K(Ca) channel's conc1 (concOut).
    Optionally `n_syn` SynChans (tau1 1 ms, tau2 3 ms, Ek 0) at random
    compartments, each driven by a Poisson train at `syn_rate`.
    `passive_props` = (Ra, Rm, Cm, area) replaces the passive values derived
    from d and L (e.g. those of a morphology loaded from a file).
    """
    n = len(parent)
    Ra, Rm, Cm, area = passive(d, L) if passive_props is None else passive_props
    (mA, mB), (hA, hB) = hh_na_tables()
    nA, nB = hh_k_tables()
    (cxA, cxB), (cyA, cyB) = ca_hva_tables()
    gates = [(VMIN, VMAX, mA, mB), (VMIN, VMAX, hA, hB), (VMIN, VMAX, nA, nB),
             (VMIN, VMAX, cxA, cxB), (VMIN, VMAX, cyA, cyB)]
    v0 = -0.065
    # channels per compartment in message order: Na, K, CaHVA
    comp = np.repeat(np.arange(n, dtype=np.uint32), 3)
    gbar = np.empty(3 * n)
    gbar[0::3] = 1200.0 * area
    gbar[1::3] = 360.0 * area
    gbar[2::3] = gca * area
    ek = np.tile([50e-3, -77e-3, ECA], n)
    xp = np.tile([3.0, 4.0, 2.0], n)
    yp = np.tile([1.0, 0.0, 1.0], n)
    xg = np.tile([0, 2, 3], n).astype(np.int32)
    yg = np.tile([1, -1, 4], n).astype(np.int32)
    X0 = np.tile([_steady(mA, mB, VMIN, VMAX, v0), _steady(nA, nB, VMIN, VMAX, v0),
                  _steady(cxA, cxB, VMIN, VMAX, v0)], n)
    Y0 = np.tile([_steady(hA, hB, VMIN, VMAX, v0), 0.0, _steady(cyA, cyB, VMIN, VMAX, v0)], n)
    tgt = np.full(3 * n, -1, np.int32)
    tgt[2::3] = np.arange(n)
    # CaConc per compartment, B from a shell of `ca_thickness`
    B = caconc_B(d, L, np.full(n, ca_thickness))
    ca_basal = 5e-5
    # K(Ca) 2-D gate
    if kca_tables is None:
        kA, kB = kca_2d_tables(cadivs=cadivs)
    else:
        kA, kB = kca_tables
    # The reference HHChannel2D has no X field: at the first reinit it sets
    # X = A/B at its default inputs (Vm = 0, conc1 = 0).  At Ca = 0 the BK
    # gate's A is 0, so X starts at 0.
    kx0 = 0.0
    m = dict(
        parent=parent, Ra=Ra, Rm=Rm, Cm=Cm, Em=np.full(n, -54.4e-3),
        initVm=np.full(n, v0), Vm=np.full(n, v0), inject=np.zeros(n),
        gates=gates, gates2d=[(VMIN, VMAX, CAMIN, CAMAX, kA, kB)],
        chan_compt=comp, chan_Gbar=gbar, chan_Ek=ek, chan_Xpower=xp, chan_Ypower=yp,
        chan_Zpower=np.zeros(3 * n), chan_xgate=xg, chan_ygate=yg,
        chan_zgate=np.full(3 * n, -1, np.int32), chan_instant=np.zeros(3 * n, np.int32),
        chan_modulation=np.ones(3 * n), chan_use_conc=np.zeros(3 * n, np.int32),
        chan_X=X0, chan_Y=Y0, chan_Z=np.zeros(3 * n), chan_ca_target=tgt,
        chan_ca_depend=np.full(3 * n, -1, np.int32),
        pool_compt=np.arange(n, dtype=np.uint32), pool_Ca=np.full(n, ca_basal),
        pool_CaBasal=np.full(n, ca_basal), pool_tau=np.full(n, 20e-3), pool_B=B,
        pool_ceiling=np.zeros(n), pool_floor=np.zeros(n),
        c2d_compt=np.arange(n, dtype=np.uint32), c2d_Gbar=gkca * area,
        c2d_Ek=np.full(n, -77e-3), c2d_Xpower=np.ones(n), c2d_xgate=np.zeros(n, np.int32),
        c2d_xindex=np.full(n, HS_DEP["VOLT_C1_INDEX"], np.int32),
        c2d_conc1_pool=np.arange(n, dtype=np.int32), c2d_conc2_pool=np.full(n, -1, np.int32),
        c2d_instant=np.zeros(n, np.int32), c2d_modulation=np.ones(n), c2d_X=np.full(n, kx0),
        sg_compt=np.array([0], np.uint32), sg_threshold=np.array([0.0]),
        sg_refractT=np.array([1e-3]), sg_edge=np.array([1], np.int32), seed=0,
        meta={"pool_diameter": d.copy(), "pool_length": L.copy(),
              "pool_thick": np.full(n, ca_thickness)})
    if inject_step:
        m.update(stim_compt=np.array([0], np.uint32), stim_step=np.array([inject_step], np.uint32),
                 stim_value=np.array([inject]))
    else:
        m["inject"][0] = inject
    if n_syn:
        rng = rng or np.random.default_rng(0)
        scomp = rng.integers(0, n, n_syn).astype(np.uint32)
        w = np.exp(rng.normal(math.log(syn_weight_median), syn_weight_sigma, n_syn))
        ev_syn, ev_time, ev_w = [], [], []
        for s in range(n_syn):
            k = rng.poisson(syn_rate * t_end)
            t = np.sort(rng.uniform(0.0, t_end, k))
            ev_syn.append(np.full(k, s, np.uint32))
            ev_time.append(t)
            ev_w.append(np.full(k, w[s]))
        m.update(syn_compt=scomp, syn_Gbar=np.ones(n_syn), syn_Ek=np.zeros(n_syn),
                 syn_tau1=np.full(n_syn, 1e-3), syn_tau2=np.full(n_syn, 3e-3),
                 syn_modulation=np.ones(n_syn),
                 ev_syn=np.concatenate(ev_syn) if ev_syn else np.zeros(0, np.uint32),
                 ev_time=np.concatenate(ev_time) if ev_time else np.zeros(0),
                 ev_weight=np.concatenate(ev_w) if ev_w else np.zeros(0))
    return CellModel(**m)


def loguniform_int(rng, lo, hi, size):
    return np.exp(rng.uniform(math.log(lo), math.log(hi), size)).round().astype(int)


def population_sizes(config, seed=1, n_cells=None):
    """Compartment counts of a workload's cells (drawn before the cells)."""
    rng = np.random.default_rng(seed)
    if config == 2:
        return rng.integers(100, 1001, n_cells or 256), 2, 0
    if config in (3, 4):
        return loguniform_int(rng, 50, 5000, n_cells or 4096), 4, (200 if config == 4 else 0)
    raise ValueError("unknown config %r" % config)


def make_cell(config, seed, i, n_cells=None, t_end=1.0, kca_tables=None, sizes=None):
    """Cell i of a workload, built alone (identical to population()[i])."""
    if sizes is None:
        sizes, maxc, nsyn = population_sizes(config, seed, n_cells)
    else:
        _, maxc, nsyn = population_sizes(config, seed, 1)
    if kca_tables is None:
        kca_tables = kca_2d_tables()
    crng = np.random.default_rng([seed, i])
    parent, d, L = branched_morphology(crng, int(sizes[i]), 0.5, maxc)
    inj = float(crng.uniform(0.1e-9, 1e-9))
    return active_cell(parent, d, L, inject=inj, n_syn=nsyn, rng=crng, t_end=t_end, kca_tables=kca_tables)


def population(config, seed=1, n_cells=None, t_end=1.0, kca_tables=None):
    """Cells of a named workload.

    config 2: 256 cells, N in [100, 1000], binary branching, 0.1-1 nA.
    config 3: 4096 cells, N log-uniform [50, 5000], junctions up to 4 children.
    config 4: config 3 cells + 200 SynChans each (5 Hz Poisson, tau1 1 ms,
              tau2 3 ms, weights lognormal median 0.5 nS).
    """
    if kca_tables is None:
        kca_tables = kca_2d_tables()
    sizes, _, _ = population_sizes(config, seed, n_cells)
    return [make_cell(config, seed, i, t_end=t_end, kca_tables=kca_tables, sizes=sizes)
            for i in range(len(sizes))]


def serving_request_work(seed, i, dt=25e-6):
    """(compartments, dt steps) of request i of the serving workload, from the
    same draws as serving_request without building the cell."""
    rng = np.random.default_rng([seed, 5, i])
    n = int(loguniform_int(rng, 100, 10000, 1)[0])
    duration = float(rng.uniform(0.1, 2.0))
    return n, int(round(duration / dt))


def serving_request(seed, i, dt=25e-6, kca_tables=None):
    """Request i of the serving workload: (cell, dt steps to simulate).

    Cells of log-uniform 100..10,000 compartments (junctions of up to 4
    children) with HH Na/K, Ca(HVA), K(Ca) and CaConc; simulated duration
    uniform 0.1..2 s; driven either by a somatic step current of 0.1..1 nA or
    by 50..500 SynChans with 5 Hz Poisson trains (even odds).
    """
    rng = np.random.default_rng([seed, 5, i])
    n = int(loguniform_int(rng, 100, 10000, 1)[0])
    duration = float(rng.uniform(0.1, 2.0))
    steps = int(round(duration / dt))
    if kca_tables is None:
        kca_tables = kca_2d_tables()
    parent, d, L = branched_morphology(rng, n, 0.5, 4)
    if rng.uniform() < 0.5:
        cell = active_cell(parent, d, L, inject=float(rng.uniform(0.1e-9, 1e-9)), rng=rng, t_end=duration,
                           kca_tables=kca_tables)
    else:
        cell = active_cell(parent, d, L, inject=0.0, n_syn=int(rng.integers(50, 501)), rng=rng, t_end=duration,
                           kca_tables=kca_tables)
    return cell, steps
