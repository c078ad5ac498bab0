"""rdesigneur's electrical cell models for the solver.

``Rdesigneur(...).build_model(t_end)`` builds, as a ``CellModel``, the cell
that the reference's ``rdesigneur.buildModel``
(``python/rdesigneur/rdesigneur.py:232-256``) hands to HSolve, from the same
arguments:

* ``cellProto`` (``buildCellProto``, ``:410-472``): ``somaProto``,
  ``ballAndStick``, ``branchedCell`` (``:495-568``), the default passive HH
  soma (``rdesigneurProtos.makePassiveHHsoma``), each compartment made as
  ``rdesigneurProtos.buildCompt`` makes it (geometry, RM/RA/CM per area,
  Em/initVm, with ``CompartmentBase``'s coordinate and length setters); or
  a passive ``CellModel`` that carries its geometry in ``meta`` (the SWC and
  GENESIS readers' models).
* ``passiveDistrib`` and ``chanDistrib``, evaluated as the C++ ``Neuron``
  class evaluates ``passiveDistribution`` and ``channelDistribution``
  (``biophysics/Neuron.cpp``): lines parsed by ``parseDistrib``
  (``:610-640``), compartments chosen by wildcard paths relative to the cell
  (``buildElist``, ``:1146-1160``), every expression evaluated per
  compartment on ``p`` (path distance from the soma), ``g`` (straight-line
  distance), ``L`` (electrotonic distance), ``len``, ``dia``, ``maxP``,
  ``maxG``, ``maxL``, ``x``, ``y``, ``z`` from the segment tree
  (``buildSegmentTree``/``updateSegmentLengths``/``traverseCumulativeDistance``,
  ``:1264-1460``; ``evalExprForElist``, ``:1530-1605``) with exprtk's
  arithmetic (``exprtk_eval``); a line's first expression selects the
  compartments (value > 0); channels copied in from the library
  (``buildFromProto``, ``:670-701``; CaConc lines first, ``:1162-1205``),
  joined to the compartment and, for a channel whose name contains ``Ca``,
  its IkOut to the compartment's CaConc (``doClassSpecificMessaging``,
  ``:642-668``) unless the prototype carries its own ``addmsg`` strings;
  fields set by ``assignParam`` (Gbar = value x len x dia x PI; Ek; a
  CaConc's geometry, CaBasal, tau, thick, floor, ceiling, ``:703-740``) and
  ``assignSingleCompartmentParams`` (RM, RA, CM per area; Rm, Ra, Cm, Em,
  initVm; ``:742-779``).
* ``stimList`` entries that set ``inject`` from an expression of ``t``
  (``_buildStims``: a ``Function`` on tick 12 with ``doEvalAtReinit``): the
  Function runs every ``funcDt`` after the solver's tick, at clock time
  ``elecDt x step`` (``scheduling/Clock.cpp:724-729``), and the solver sees
  its value from the next step on; this becomes the model's stimulus
  schedule.

The channel library (rdesigneur's ``chanProto``, made by
``rdesigneurProtos`` functions in the reference) is a dict of the
``genesis`` prototype classes (``HHChannelProto``, ``HHChannel2DProto``,
``SynChanProto`` -- ``make_glu`` and the like; ``assignParam`` treats a
SynChan as every ChanBase: Gbar per area, Ek -- and ``CaConcProto``),
each with a ``Gbar`` attribute for the prototype's own Gbar (kept where a
distribution does not set it).  SynChans get no events from the loader
(the model's ``ev_*`` arrays, or ``hs_push_events`` at run time).  The HSolve target is the
largest-diameter compartment whose name contains ``oma``, as rdesigneur
picks its soma.  Not built: spines, chemistry, adaptors, plots, other
stimulus kinds.
"""
import math
import re

import numpy as np

from . import genesis
from .abi import CellModel
from .exprtk_eval import Expression

PI_PROTOS = 3.14159265359      # rdesigneurProtos.PI (buildCompt)
PI = 3.141592653589793         # basecode/header.h PI (Neuron)
FARADAY = 96485.3415           # basecode/header.h FaradayConst
VALENCE = 2.0                  # CaConcBase VALENCE


class Compartment:
    """One compartment as buildCompt and the distributions leave it."""

    def __init__(self, name, parent):
        self.name, self.parent = name, parent
        self.x0 = self.y0 = self.z0 = self.x = self.y = self.z = 0.0
        self.dia = self.length = 0.0
        self.Ra = self.Rm = self.Cm = 0.0
        self.Em = self.initVm = -0.065
        self.objs = []                 # (name, proto, fields), creation order

    def set_geometry(self, x0, y0, z0, x, y, z, dia, length):
        """CompartmentBase setters in buildCompt's order: x0, y0, z0, x, y,
        z (each recomputing length_), diameter, then setLength, which
        rescales the end point when the coordinates agree with length_
        (biophysics/CompartmentBase.cpp:488-512)."""
        cur = math.sqrt((x - x0) * (x - x0) + (y - y0) * (y - y0) + (z - z0) * (z - z0))
        if length > 0 and cur > 0 and genesis._double_eq(cur * cur, (x - x0) * (x - x0) + (y - y0) * (y - y0)
                                                          + (z - z0) * (z - z0)):
            ratio = length / cur
            x = x0 + ratio * (x - x0)
            y = y0 + ratio * (y - y0)
            z = z0 + ratio * (z - z0)
        self.x0, self.y0, self.z0, self.x, self.y, self.z = x0, y0, z0, x, y, z
        self.dia, self.length = dia, length

    def child(self, name):
        return next((o for o in self.objs if o[0] == name), None)


def build_compt(cell, name, parent=None, RM=1.0, RA=1.0, CM=0.01, dia=1.0e-6, x=0.0, y=0.0, z=0.0, dx=10e-6,
                dy=0.0, dz=0.0, Em=-0.065, initVm=-0.065):
    """rdesigneurProtos.buildCompt (python/rdesigneur/rdesigneurProtos.py:620-638)."""
    length = math.sqrt(dx * dx + dy * dy + dz * dz)
    c = Compartment(name, parent)
    c.set_geometry(x, y, z, dx + x, dy + y, dz + z, dia, length)
    xa = dia * dia * PI_PROTOS / 4.0
    sa = length * dia * PI_PROTOS
    c.Ra = length * RA / xa
    c.Rm = RM / sa
    c.Cm = CM * sa
    c.Em, c.initVm = Em, initVm
    cell.append(c)
    return c


# ---- cell prototypes (rdesigneur.py:495-568) -----------------------------------
def soma_proto(args):
    parms = ["somaProto", "soma", 5e-4, 5e-4]
    parms[:len(args)] = args
    cell = []
    build_compt(cell, "soma", dia=parms[2], dx=parms[3])
    return cell


def ball_and_stick(args):
    parms = ["ballAndStick", "cell", 10e-6, 10e-6, 4e-6, 200e-6, 1]
    parms[:len(args)] = args
    if parms[6] <= 0:
        return soma_proto(parms[:4])
    cell = []
    prev = build_compt(cell, "soma", dia=args[2], dx=args[3])
    dx = parms[5] / parms[6]
    x = prev.x
    for i in range(parms[6]):
        prev = build_compt(cell, "dend" + str(i), parent=len(cell) - 1, x=x, dx=dx, dia=args[4])
        x += dx
    return cell


def branched_cell(args):
    parms = ["branchedCell", "cell", 10e-6, 10e-6, 4e-6, 200e-6, 1, 2.5e-6, 200e-6, 1]
    parms[:len(args)] = args
    if parms[9] <= 0:
        return soma_proto(parms[:4])
    cell = []
    prev = build_compt(cell, "soma", dia=args[2], dx=args[3])
    dx = parms[5] / parms[6]
    x = prev.x
    for i in range(parms[6]):
        prev = build_compt(cell, "dend" + str(i), parent=len(cell) - 1, x=x, dx=dx, dia=args[4])
        x += dx
    end = len(cell) - 1
    dxy = (parms[8] / float(parms[9])) * math.sqrt(1.0 / 2.0)
    for branch, sign in (("branch1_", 1.0), ("branch2_", -1.0)):
        x, y = cell[end].x, cell[end].y
        pa = end
        for i in range(parms[9]):
            build_compt(cell, branch + str(i), parent=pa, x=x, dx=dxy, y=y, dy=sign * dxy, dia=args[7])
            pa = len(cell) - 1
            x += dxy
            y += sign * dxy
    return cell


def passive_hh_soma():
    """rdesigneurProtos.makePassiveHHsoma: a 500 um squid-sized soma."""
    cell = []
    soma = build_compt(cell, "soma", dx=500e-6, dia=500e-6, x=0.0, RM=0.33333333, RA=3000, CM=0.01)
    soma.initVm = -65e-3
    soma.Em = -54.4e-3
    return cell


def from_model(m):
    """A passive CellModel with geometry in meta (names, coords, diameter,
    length) as a cell prototype."""
    if len(m.chan_compt) or len(m.pool_compt) or len(m.c2d_compt) or len(m.syn_compt):
        raise ValueError("rdesigneur cell prototype from a model: only passive models (channels come from "
                         "chanDistrib)")
    for key in ("names", "coords", "diameter", "length"):
        if key not in m.meta:
            raise ValueError("rdesigneur cell prototype from a model: meta[%r] missing" % key)
    cell = []
    for i in range(m.n_compt):
        c = Compartment(str(m.meta["names"][i]), int(m.parent[i]) if m.parent[i] >= 0 else None)
        x0, y0, z0, x, y, z = (float(v) for v in m.meta["coords"][i])
        c.x0, c.y0, c.z0, c.x, c.y, c.z = x0, y0, z0, x, y, z
        c.dia, c.length = float(m.meta["diameter"][i]), float(m.meta["length"][i])
        c.Ra, c.Rm, c.Cm = float(m.Ra[i]), float(m.Rm[i]), float(m.Cm[i])
        c.Em, c.initVm = float(m.Em[i]), float(m.initVm[i])
        cell.append(c)
    return cell


# ---- the Neuron's segment tree --------------------------------------------------
class SegmentTree:
    """Neuron::buildSegmentTree + updateSegmentLengths: per compartment its
    path (p), straight-line (g) and electrotonic (L) distance from the
    first compartment, and their maxima."""

    def __init__(self, cell):
        n = len(cell)
        self.p = [0.0] * n
        self.g = [0.0] * n
        self.L = [0.0] * n
        kids = [[] for _ in range(n)]
        for i, c in enumerate(cell):
            if c.parent is not None:
                kids[c.parent].append(i)
        v = [(c.x, c.y, c.z) for c in cell]

        def dist(a, b):
            d0, d1, d2 = a[0] - b[0], a[1] - b[1], a[2] - b[2]
            return math.sqrt(d0 * d0 + d1 * d1 + d2 * d2)
        for i in range(n):
            self.g[i] = dist(v[i], v[0])
        stack = [(0, 0.0, 0.0)]
        while stack:
            i, p, e = stack.pop()
            self.p[i], self.L[i] = p, e
            for k in reversed(kids[i]):
                seg = dist(v[k], v[i])
                stack.append((k, p + seg, e + math.sqrt(cell[k].Ra / cell[k].Rm)))
        self.maxP, self.maxG, self.maxL = 0.0, 0.0, 0.0
        for i in range(n):
            self.maxP = max(self.maxP, self.p[i])
            self.maxG = max(self.maxG, self.g[i])
            self.maxL = max(self.maxL, self.L[i])
        self.v = v

    def values(self, cell, i):
        """nuParser's variables for compartment i (evalExprForElist)."""
        c = cell[i]
        return dict(p=self.p[i], g=self.g[i], L=self.L[i], len=c.length, dia=c.dia, maxP=self.maxP,
                    maxG=self.maxG, maxL=self.maxL, x=self.v[i][0], y=self.v[i][1], z=self.v[i][2],
                    oldVal=0.0)


def select(cell, path):
    """The compartments a wildcard path relative to the cell names, in
    creation order: comma-separated patterns of names where ``#`` matches
    any run of characters and ``?`` one, optionally ``[ISA=...]`` or
    ``[TYPE=...]`` naming a compartment class; ``##`` (any depth) is the same
    as ``#`` for a cell's compartments."""
    out = set()
    for pat in path.split(","):
        pat = pat.strip()
        m = re.fullmatch(r"(.*?)(\[(ISA|TYPE)=(\w+)\])?", pat)
        name, cls = m.group(1), m.group(4)
        if cls is not None and cls not in ("CompartmentBase", "Compartment", "SymCompartment"):
            continue
        name = name.replace("##", "#")
        if "/" in name:
            raise ValueError("rdesigneur paths below the cell's compartments are not built: %r" % pat)
        rx = re.compile("^" + "".join(".*" if ch == "#" else "." if ch == "?" else re.escape(ch)
                                      for ch in name) + "$")
        out.update(i for i, c in enumerate(cell) if rx.match(c.name))
    return sorted(out)


def parse_distrib(flat):
    """Neuron's parseDistrib: lines separated by "" entries, each of at
    least 4 and an even number of entries."""
    lines, cur = [], []
    for s in flat:
        if s == "":
            if len(cur) < 4 or len(cur) % 2 == 1:
                raise ValueError("distribution line %r: needs 4 or more, and an even number of, entries" % cur)
            lines.append(cur)
            cur = []
        else:
            cur.append(s)
    return lines


class Rdesigneur:
    """The electrical part of rdesigneur's model, for the solver."""

    def __init__(self, cellProto=(), library=None, passiveDistrib=(), chanDistrib=(), stimList=(),
                 elecDt=50e-6, funcDt=100e-6):
        self.cellProto = list(cellProto)
        self.library = dict(library or {})
        self.passiveDistrib = [list(x) for x in passiveDistrib]
        self.chanDistrib = [list(x) for x in chanDistrib]
        self.stimList = [list(x) for x in stimList]
        self.elecDt, self.funcDt = float(elecDt), float(funcDt)

    # -- cell
    def _cell(self):
        if not self.cellProto:
            return passive_hh_soma()
        cell = None
        for proto in self.cellProto:
            kind = proto[0]
            if isinstance(kind, CellModel):
                cell = from_model(kind)
            elif kind == "somaProto":
                cell = soma_proto(list(proto))
            elif kind == "ballAndStick":
                cell = ball_and_stick(list(proto))
            elif kind == "branchedCell":
                cell = branched_cell(list(proto))
            else:
                raise ValueError("cellProto %r: not built (somaProto, ballAndStick, branchedCell or a "
                                 "CellModel)" % (kind,))
        return cell

    def _line_values(self, cell, tree, idx, expr):
        f = Expression(expr)
        return [f(**tree.values(cell, i)) for i in idx]

    # -- Neuron::setPassiveDistribution
    def _passive(self, cell, tree):
        flat = []
        for line in self.passiveDistrib:
            if len(line) < 3 or (line[0] != "." and len(line) % 2 != 1):
                raise ValueError("passiveDistrib: need path field expr [field expr]..., have %r" % line)
            if not (len(line) % 2 != 1 and line[0] == "."):
                flat.append(".")
            flat += line + [""]
        for line in parse_distrib(flat):
            idx = select(cell, line[1])
            sel = self._line_values(cell, tree, idx, line[3])
            for j in range(2, len(line), 2):
                field, vals = line[j], self._line_values(cell, tree, idx, line[j + 1])
                for i, s, x in zip(idx, sel, vals):
                    if s > 0:
                        _assign_compartment(cell[i], field, x)

    # -- Neuron::setChannelDistribution
    def _channels(self, cell, tree):
        flat = []
        for line in self.chanDistrib:
            flat += list(line) + [""]
        lines = parse_distrib(flat)
        for line in lines:
            if line[0] not in self.library:
                raise ValueError("chanDistrib: prototype %r is not in the library" % line[0])
        ca = [ln for ln in lines if isinstance(self.library[ln[0]], genesis.CaConcProto)]
        lines = ca + [ln for ln in lines if not isinstance(self.library[ln[0]], genesis.CaConcProto)]
        for line in lines:
            proto = self.library[line[0]]
            idx = select(cell, line[1])
            sel = self._line_values(cell, tree, idx, line[3])
            mech = {}
            for i, s in zip(idx, sel):
                if s > 0:
                    obj = cell[i].child(line[0])
                    if obj is None:
                        obj = (line[0], proto, _initial_fields(proto))
                        cell[i].objs.append(obj)
                        _class_messages(cell[i], obj)
                    mech[i] = obj
            for j in range(2, len(line), 2):
                field, vals = line[j], self._line_values(cell, tree, idx, line[j + 1])
                for i, s, x in zip(idx, sel, vals):
                    if s > 0:
                        _assign_param(mech[i], field, x, cell[i].length, cell[i].dia)

    # -- stimulus: inject Functions on tick 12
    def _stims(self, cell, tree, nsteps):
        k = max(1, int(round(self.funcDt / self.elecDt)))
        sched = {}
        inject0 = {}
        for st in self.stimList:
            if len(st) < 5 or st[3] != "inject":
                raise ValueError("stimList: only 'inject' entries are built, got %r" % (st,))
            idx = select(cell, st[0])
            geom = self._line_values(cell, tree, idx, st[1])
            f = Expression(st[4])
            for i, gv in zip(idx, geom):
                if gv <= 0:
                    continue
                inject0[i] = f(t=0.0)
                prev = inject0[i]
                for s in range(1, nsteps):
                    e = s - s % k
                    val = f(t=self.elecDt * e) if e else inject0[i]
                    if val != prev:
                        sched.setdefault(s, []).append((i, val))
                        prev = val
        return inject0, sched

    def build_model(self, t_end=0.0, seed=None):
        """The CellModel HSolve would get, with the stimulus schedule for
        t_end seconds at elecDt."""
        cell = self._cell()
        tree = SegmentTree(cell)
        self._passive(cell, tree)
        self._channels(cell, tree)
        nsteps = int(round(t_end / self.elecDt)) if t_end > 0 else 0
        inject0, sched = self._stims(cell, tree, max(nsteps, 1))
        somas = [i for i, c in enumerate(cell) if "oma" in c.name]
        if seed is None:
            seed = max(somas, key=lambda i: cell[i].dia) if somas else 0
        return _to_model(cell, seed, inject0, sched)


def _initial_fields(proto):
    f = {"Gbar": float(getattr(proto, "Gbar", 0.0))}
    if isinstance(proto, genesis.CaConcProto):
        f.update(tau=proto.tau, CaBasal=proto.CaBasal, thick=proto.thick, diameter=proto.diameter,
                 length=proto.length, ceiling=proto.ceiling, floor=proto.floor)
    else:
        f["Ek"] = proto.Ek
    return f


def _class_messages(c, obj):
    """doClassSpecificMessaging: a channel whose name contains "Ca" sends
    IkOut to the compartment's first CaConc, unless the prototype has its
    own addmsg strings; then the prototype's addmsg strings
    (ReadCell::addChannelMessage, biophysics/ReadCell.cpp:984-1031): a
    message whose source or destination the compartment does not hold
    (yet) is skipped, as there."""
    name, proto, f = obj
    if isinstance(proto, genesis.CaConcProto):
        return
    addmsg = list(getattr(proto, "addmsg", ()))
    pools = [o[0] for o in c.objs if isinstance(o[1], genesis.CaConcProto)]
    if "Ca" in name and not addmsg and pools:
        f["ca_target"] = pools[0]
    for m in addmsg:
        src, sf, dst, df = m.split()
        rel = lambda p: name if p == "." else p[3:] if p.startswith("../") else None
        s, d = rel(src), rel(dst)
        exists = lambda x: x == name or x in pools
        if s is None or d is None or not exists(s) or not exists(d):
            continue
        if s == name and sf == "IkOut" and df == "current":
            f.setdefault("ca_target", d)
        elif d == name and sf == "concOut" and df in ("concen", "concen1"):
            f["ca_depend"] = s
        elif d == name and sf == "concOut" and df == "concen2":
            f["conc2"] = s
        else:
            raise ValueError("addmsg %r of %s: only IkOut->current and concOut->concen are built" % (m, name))


def _assign_param(obj, field, x, length, dia):
    """Neuron.cpp assignParam."""
    name, proto, f = obj
    if isinstance(proto, genesis.CaConcProto):
        f["length"], f["diameter"] = length, dia
        if field in ("CaBasal", "tau", "thick", "floor", "ceiling"):
            f[field] = x
        return
    if field == "Gbar":
        if x > 0:
            f["Gbar"] = x * length * dia * PI
    elif field == "Ek":
        f["Ek"] = x


def _assign_compartment(c, field, x):
    """Neuron.cpp assignSingleCompartmentParams."""
    if field in ("initVm", "INITVM"):
        c.initVm = x
        return
    if field in ("Em", "EM"):
        c.Em = x
        return
    if x > 0.0:
        if field == "Rm":
            c.Rm = x
        elif field == "Ra":
            c.Ra = x
        elif field == "Cm":
            c.Cm = x
        elif field == "RM":
            c.Rm = x / (c.length * c.dia * PI)
        elif field == "RA":
            c.Ra = x * c.length * 4 / (c.dia * c.dia * PI)
        elif field == "CM":
            c.Cm = x * c.length * c.dia * PI
        else:
            raise ValueError("passiveDistrib: field %r is not a compartment parameter" % field)


def _pool_B(f):
    """B as zombification leaves it (CaConcBase::updateDimensions)."""
    vol = PI * f["diameter"] * f["diameter"] * f["length"] * 0.25
    if 0 < f["thick"] < f["diameter"] / 2.0:
        core = f["diameter"] / 2.0 - f["thick"]
        vol -= PI * core * core * f["length"]
    return 1.0 / (VALENCE * FARADAY * vol)


def _to_model(cell, seed, inject0, sched):
    gates, gate_ix = [], {}
    gates2d, gate2d_ix = [], {}

    def gate(pname, letter, g):
        key = (pname, letter)
        if key not in gate_ix:
            gate_ix[key] = len(gates)
            gates.append((float(g[0]), float(g[1]), np.asarray(g[2], float), np.asarray(g[3], float)))
        return gate_ix[key]

    pools, pool_of = [], []
    for i, c in enumerate(cell):
        names = {}
        for name, proto, f in c.objs:
            if isinstance(proto, genesis.CaConcProto):
                names[name] = len(pools)
                pools.append((i, f))
        pool_of.append(names)
    ch, c2, sy = [], [], []
    for i, c in enumerate(cell):
        for name, proto, f in c.objs:
            if isinstance(proto, genesis.HHChannelProto):
                ch.append((i, name, proto, f))
            elif isinstance(proto, genesis.HHChannel2DProto):
                c2.append((i, name, proto, f))
            elif isinstance(proto, genesis.SynChanProto):
                sy.append((i, name, proto, f))
    f64 = lambda v: np.asarray(v, np.float64)
    i32 = lambda v: np.asarray(v, np.int32)
    u32 = lambda v: np.asarray(v, np.uint32)
    for i, name, p, f in c2:
        if name not in gate2d_ix:
            gate2d_ix[name] = len(gates2d)
            xmn, xmx, ymn, ymx, A, B = p.table
            gates2d.append((float(xmn), float(xmx), float(ymn), float(ymx), np.asarray(A, float),
                            np.asarray(B, float)))
    n, nc, n2 = len(cell), len(ch), len(c2)
    steps = sorted(sched)
    stim = [(s, i, v) for s in steps for i, v in sched[s]]
    from .abi import HS_DEP
    return CellModel(
        seed=seed, gates=gates, gates2d=gates2d,
        parent=i32([-1 if c.parent is None else c.parent for c in cell]),
        Ra=f64([c.Ra for c in cell]), Rm=f64([c.Rm for c in cell]), Cm=f64([c.Cm for c in cell]),
        Em=f64([c.Em for c in cell]), initVm=f64([c.initVm for c in cell]), Vm=f64([c.initVm for c in cell]),
        inject=f64([inject0.get(i, 0.0) for i in range(n)]),
        chan_compt=u32([r[0] for r in ch]), chan_Gbar=f64([r[3]["Gbar"] for r in ch]),
        chan_Ek=f64([r[3]["Ek"] for r in ch]),
        chan_Xpower=f64([r[2].Xpower for r in ch]), chan_Ypower=f64([r[2].Ypower for r in ch]),
        chan_Zpower=f64([r[2].Zpower for r in ch]),
        chan_xgate=i32([gate(r[1], "X", r[2].xgate) if r[2].Xpower > 0 else -1 for r in ch]),
        chan_ygate=i32([gate(r[1], "Y", r[2].ygate) if r[2].Ypower > 0 else -1 for r in ch]),
        chan_zgate=i32([gate(r[1], "Z", r[2].zgate) if r[2].Zpower > 0 else -1 for r in ch]),
        chan_instant=i32([r[2].instant for r in ch]), chan_modulation=np.ones(nc),
        chan_use_conc=i32([r[2].useConcentration for r in ch]),
        chan_X=np.zeros(nc), chan_Y=np.zeros(nc), chan_Z=np.zeros(nc),
        chan_ca_target=i32([pool_of[r[0]][r[3]["ca_target"]] if "ca_target" in r[3] else -1 for r in ch]),
        chan_ca_depend=i32([pool_of[r[0]][r[3]["ca_depend"]] if "ca_depend" in r[3] else -1 for r in ch]),
        pool_compt=u32([p[0] for p in pools]), pool_Ca=f64([p[1]["CaBasal"] for p in pools]),
        pool_CaBasal=f64([p[1]["CaBasal"] for p in pools]), pool_tau=f64([p[1]["tau"] for p in pools]),
        pool_B=f64([_pool_B(p[1]) for p in pools]), pool_ceiling=f64([p[1]["ceiling"] for p in pools]),
        pool_floor=f64([p[1]["floor"] for p in pools]),
        c2d_compt=u32([r[0] for r in c2]), c2d_Gbar=f64([r[3]["Gbar"] for r in c2]),
        c2d_Ek=f64([r[3]["Ek"] for r in c2]), c2d_Xpower=f64([r[2].Xpower for r in c2]),
        c2d_xgate=i32([gate2d_ix[r[1]] for r in c2]), c2d_xindex=i32([HS_DEP[r[2].Xindex] for r in c2]),
        c2d_conc1_pool=i32([pool_of[r[0]][r[3]["ca_depend"]] if "ca_depend" in r[3] else -1 for r in c2]),
        c2d_conc2_pool=i32([pool_of[r[0]][r[3]["conc2"]] if "conc2" in r[3] else -1 for r in c2]),
        c2d_instant=np.zeros(n2, np.int32), c2d_modulation=np.ones(n2), c2d_X=np.zeros(n2),
        syn_compt=u32([r[0] for r in sy]), syn_Gbar=f64([r[3]["Gbar"] for r in sy]),
        syn_Ek=f64([r[3]["Ek"] for r in sy]), syn_tau1=f64([r[2].tau1 for r in sy]),
        syn_tau2=f64([r[2].tau2 for r in sy]), syn_modulation=np.ones(len(sy)),
        ev_syn=np.zeros(0, np.uint32), ev_time=np.zeros(0), ev_weight=np.zeros(0),
        stim_compt=u32([s[1] for s in stim]), stim_step=u32([s[0] for s in stim]),
        stim_value=f64([s[2] for s in stim]),
        meta={"names": [c.name for c in cell], "diameter": f64([c.dia for c in cell]),
              "length": f64([c.length for c in cell]),
              "coords": f64([(c.x0, c.y0, c.z0, c.x, c.y, c.z) for c in cell]).reshape(-1, 6),
              "chan_name": [r[1] for r in ch], "syn_name": [r[1] for r in sy]})
