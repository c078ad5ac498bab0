"""GENESIS .p cell reader: compartmental cells for the solver from GENESIS
cell files, built the way MOOSE's ``ReadCell`` builds them
(``biophysics/ReadCell.cpp``, called by ``loadModel`` for ``.p`` files,
``shell/LoadModels.cpp:148-153``).

The channel library -- MOOSE's ``/library`` of prototype objects that a .p
file names -- is a dict of the prototype classes below (HHChannelProto,
HHChannel2DProto, SynChanProto, CaConcProto, SpikeGenProto, and
CompartmentProto for ``*compt``).  A prototype's ``addmsg``
strings are GENESIS ``addmsg`` fields (``"src srcField dest destField"``,
``.`` the object itself, ``../NAME`` a sibling in the same compartment),
resolved after each line's channels are made, as
``ReadCell::addChannelMessage`` does (``ReadCell.cpp:984-1031``).

Followed step by step, in the reference's operation order so that passive
values and coordinates come out bit for bit:
  * ``innerRead`` (``ReadCell.cpp:154-218``): trimmed lines, ``//`` comments
    (whole line or tail), ``/* ... */`` blocks (a line inside a block that
    starts with ``*`` is read as a command, as in the reference), ``*``
    commands, data lines;
  * ``readScript`` (``:220-306``): ``*cartesian``/``*polar``,
    ``*relative``/``*absolute``, ``*symmetric``/``*asymmetric``, ``*set_global`` /
    ``*set_compt_param`` RM RA CM EREST_ACT ELEAK, ``*start_cell``,
    ``*double_endpoint``/``*double_endpoint_off``, ``*makeproto``;
  * ``readData`` (``:308-375``): coordinates in um (polar: r, theta and phi
    in degrees), diameter;
  * ``buildCompartment`` (``:377-555``): ``.`` = the previous compartment,
    ``none``/``nil`` = a root; start point = the parent's end point
    (relative coordinates add it); length from the start point (a root
    without a start point: from the origin; length 0 = a sphere);
    Cm = CM surf, Rm = RM/surf, Ra = RA len 4/(d^2 pi) (a sphere:
    RA 8/(d pi)); Em / initVm from ELEAK / EREST_ACT by which was set; the
    coordinates end as ``CompartmentBase::setLength`` leaves them;
  * ``buildChannels`` (``:628-735``): ``RA RM CM`` scale by the geometry
    (RM multiplies by the surface, as in the reference), ``Ra Rm Cm`` are
    absolute, ``kinModel``/``m2c``/``c2m`` take their arguments and do
    nothing; a channel's Gbar = value x surface (value > 0) or -value; a
    CaConc's value is scaled by its shell volume; a SpikeGen's value is its
    threshold.
The solver then sees a CaConc's B as zombification leaves it: recomputed
from the CaConc's thick, length and diameter (``CaConcBase::zombify``,
``updateDimensions``, ``CaConcBase.cpp:259-269, 347-391``), i.e. the
prototype's geometry, not the compartment's.

Symmetric cells (``*symmetric``): the compartments are SymCompartments,
joined to their parent by a ``distal`` -> ``proximal`` message and, as
``ReadCell.cpp:501-510`` does, to every object the parent's ``distalOut``
already reaches (its earlier children and its own siblings) by ``sibling``
messages.  HSolve reads a SymCompartment exactly as a Compartment (same
fields, same matrix: ``HSolve.cpp:505-513``, ``HSolvePassive.cpp:100-165``),
so an unbranched symmetric cell solves to the same numbers as the
asymmetric one.  A ``sibling`` message carries ``distalOut``, which
``HSolveUtils::adjacent`` (``HSolveUtils.cpp:36-45``) follows, so the
reference's tree walk (``HSolvePassive::walkTree``) never ends on a cell
with sibling messages; such a model is loaded with its sibling links in
``meta["sibling_links"]`` and ``CellModel.desc()`` refuses it (ValueError)
instead of describing a tree the reference cannot set up.  A symmetric
compartment on a non-symmetric parent is rejected (ValueError): ReadCell's
``distal`` message needs a SymCompartment at both ends.

Compartment prototypes (``*compt <path>``, ``ReadCell.cpp:274-291,
447-470``): from that line on, each compartment is a copy of the
prototype (``Shell::doCopy``): its child objects with their own field
values (a channel's Gbar as set in the prototype, not scaled), the
messages among them, and its inject; then the line's geometry, passive
values and channels apply as for a plain compartment, the line's channels
after the prototype's.  A prototype is a ``CompartmentProto`` in the
library; ``*compt`` takes it only when the path equals the prototype's
``Id::path()`` -- ``/library[0]/NAME`` for the library entry ``NAME``
(``Neutral::path`` puts ``[0]`` on every element but the last, and
``Id::path`` trims only the last) -- and otherwise warns and keeps the
previous prototype, as the reference's path check does.

Not supported (ValueError): grafted cells (``*start_cell path``), a
compartment prototype whose class (Compartment or SymCompartment) differs
from ``*symmetric``/``*asymmetric`` (ReadCell's messages would not join
it to its parent), ``addmsg`` wiring other than IkOut->current and
concOut->concen/concen2.
"""
import math
import re

import numpy as np

from .abi import HS_DEP, CellModel
from .swc import _atof

M_PI = 3.141592653589793
# CaConcBase::updateDimensions: B = 1/(VALENCE FaradayConst vol) (basecode/header.h)
_PI_MOOSE = 3.141592653589793
_FARADAY = 96485.3415
_VALENCE = 2.0


class HHChannelProto:
    """An HHChannel prototype: Ek, gate powers, gate tables (min, max, A, B)
    with len(A) = divs + 1, useConcentration for the Z gate, addmsg."""

    def __init__(self, Ek, Xpower=0, Ypower=0, Zpower=0, xgate=None, ygate=None, zgate=None, instant=0,
                 useConcentration=0, addmsg=()):
        self.Ek, self.instant, self.useConcentration = Ek, instant, useConcentration
        self.Xpower, self.Ypower, self.Zpower = Xpower, Ypower, Zpower
        self.xgate, self.ygate, self.zgate = xgate, ygate, zgate
        self.addmsg = list(addmsg)


class HHChannel2DProto:
    """An HHChannel2D prototype: Ek, Xpower, Xindex (e.g. VOLT_C1_INDEX) and
    its 2-D table (xmin, xmax, ymin, ymax, A[x][y], B[x][y])."""

    def __init__(self, Ek, Xpower, table, Xindex="VOLT_C1_INDEX", addmsg=()):
        self.Ek, self.Xpower, self.table, self.Xindex = Ek, Xpower, table, Xindex
        self.addmsg = list(addmsg)


class SynChanProto:
    """A SynChan prototype (Ek, tau1, tau2) with its SimpleSynHandler of one
    synapse of the given weight, as ``rdesigneurProtos.make_glu`` builds
    one.  ReadCell adds it as it adds an HHChannel (``addCanonicalChannel``,
    ``ReadCell.cpp:773-800``: the ``channel`` message and Gbar).  The
    loader queues no events: they are the model's ``ev_*`` arrays, or
    arrive at run time (``hs_push_events``)."""

    def __init__(self, Ek, tau1, tau2, weight=1.0, addmsg=()):
        self.Ek, self.tau1, self.tau2, self.weight = Ek, tau1, tau2, weight
        self.addmsg = list(addmsg)


class CaConcProto:
    """A CaConc prototype (tau, CaBasal, shell thick, diameter, length,
    ceiling, floor)."""

    def __init__(self, tau, CaBasal, thick, diameter, length, ceiling=0.0, floor=0.0, addmsg=()):
        self.tau, self.CaBasal, self.thick = tau, CaBasal, thick
        self.diameter, self.length, self.ceiling, self.floor = diameter, length, ceiling, floor
        self.addmsg = list(addmsg)

    def zombie_B(self):
        """B after HSolve zombifies the pool (updateDimensions on the
        object's own geometry)."""
        d, L, t = self.diameter, self.length, self.thick
        vol = _PI_MOOSE * d * d * L * 0.25
        if t > 0 and t < d / 2.0:
            core = d / 2.0 - t
            vol -= _PI_MOOSE * core * core * L
        return 1.0 / (_VALENCE * _FARADAY * vol)


class SpikeGenProto:
    def __init__(self, refractT=0.0, edgeTriggered=1, addmsg=()):
        self.refractT, self.edgeTriggered = refractT, edgeTriggered
        self.addmsg = list(addmsg)


class CompartmentProto:
    """A compartment prototype for ``*compt``: the copied compartment's
    children as (name, prototype, fields) in the order of the compartment's
    messages to them (a channel's ``Gbar``, absolute; a SpikeGen's
    ``threshold``; a CaConc needs none), the messages among them as
    (src, srcField, dst, dstField) with IkOut -> current and concOut ->
    concen/concen2, the compartment's inject, and its class."""

    def __init__(self, children=(), msgs=(), inject=0.0, symmetric=False):
        self.children = [(n, p, dict(f)) for n, p, f in children]
        self.msgs = [tuple(m) for m in msgs]
        self.inject = inject
        self.symmetric = bool(symmetric)


def proto_path(name):
    """``Id::path()`` of a library entry: every element but the last with
    its ``[0]`` (``/library[0]/NAME``); a name given as an absolute path is
    taken as the element's path."""
    parts = name.strip("/").split("/") if name.startswith("/") else ["library", name]
    return "/" + "".join(p + "[0]/" for p in parts[:-1]) + parts[-1]


def calc_surf(length, dia):
    """calcSurf (ReadCell.cpp:617-626): a sphere when length is 0."""
    return dia * dia * M_PI if length == 0.0 else length * dia * M_PI


def _double_eq(x, y):
    """doubleEq (basecode/doubleEq.cpp:16-22)."""
    denom = abs(x) + abs(y)
    if denom < 1e-12:
        denom = 1e-6
    return abs(x - y) / denom < 1e-6


_WS = re.compile(r"[\t ]+")


def _tokens(line):
    return [t for t in _WS.split(line) if t]


class _Compt:
    __slots__ = ("name", "parent", "x0", "y0", "z0", "x", "y", "z", "d", "length", "Rm", "Ra", "Cm",
                 "initVm", "Em", "objs", "sym", "distal", "sibs", "inject")


class ReadCell:
    """One .p file read into compartments and their channel objects."""

    def __init__(self, library):
        self.lib = dict(library)
        self.RM, self.CM, self.RA = 10.0, 0.01, 1.0
        self.EREST_ACT, self.ELEAK = -0.065, -0.065
        self.erest_flag = self.eleak_flag = 0
        self.polar = self.relative = self.double_endpoint = self.symmetric = 0
        self.proto = None
        self.compts = []
        self.by_name = {}
        self.last = None
        self.warnings = []
        self.line_num = 0

    # ---- innerRead
    def read(self, text):
        mode = "DATA"
        for raw in text.split("\n"):
            line = raw.strip(" \t\r\n")
            self.line_num += 1
            if not line:
                continue
            if line[:2] == "//":
                continue
            pos = line.find("//")
            if pos >= 0:
                line = line[:pos]
            if line[:2] == "/*":
                mode = "COMMENT"
            elif "*/" in line:
                mode = "DATA"
                continue
            elif line[0] == "*":
                mode = "SCRIPT"
            if mode == "COMMENT":
                pos = line.find("*/")
                if pos >= 0:
                    mode = "DATA"
                    if len(line) > pos + 2:
                        line = line[pos + 2:]
            if mode == "DATA":
                self._data(line)
            elif mode == "SCRIPT":
                self._script(line)
                mode = "DATA"
        return self

    def _warn(self, msg):
        self.warnings.append("line %d: %s" % (self.line_num, msg))

    # ---- readScript
    def _script(self, line):
        argv = _tokens(line)
        c = argv[0] if argv else ""
        if c == "*cartesian":
            self.polar = 0
        elif c == "*polar":
            self.polar = 1
        elif c == "*relative":
            self.relative = 1
        elif c == "*absolute":
            self.relative = 0
        elif c == "*symmetric":
            self.symmetric = 1
        elif c == "*asymmetric":
            self.symmetric = 0
        elif c in ("*set_global", "*set_compt_param"):
            if len(argv) != 3:
                self._warn("bad line")
                return
            v = _atof(argv[2])
            if argv[1] == "RM":
                self.RM = v
            if argv[1] == "RA":
                self.RA = v
            if argv[1] == "CM":
                self.CM = v
            if argv[1] == "EREST_ACT":
                self.EREST_ACT, self.erest_flag = v, 1
            if argv[1] == "ELEAK":
                self.ELEAK, self.eleak_flag = v, 1
        elif c == "*start_cell":
            if len(argv) != 1:
                raise ValueError("grafted cells (*start_cell <path>) are not supported")
        elif c == "*compt":
            if len(argv) != 2:
                self._warn("bad line")
                return
            for key, p in self.lib.items():
                if isinstance(p, CompartmentProto) and proto_path(key) == argv[1]:
                    self.proto = p
                    break
            else:
                self._warn("bad path: %s" % argv[1])
        elif c == "*double_endpoint":
            self.double_endpoint = 1
        elif c == "*double_endpoint_off":
            self.double_endpoint = 0
        elif c == "*makeproto":
            pass
        else:
            self._warn("command %s not recognized, ignored" % c)

    # ---- readData
    def _data(self, line):
        argv = _tokens(line)
        if len(argv) < 6:
            self._warn("too few arguments (%d)" % len(argv))
            return
        x0 = y0 = z0 = 0.0
        off = 0
        if self.double_endpoint:
            if len(argv) < 9:
                raise ValueError("line %d: a double-endpoint line needs 9 fields" % self.line_num)
            off = 3
            x0 = 1.0e-6 * _atof(argv[2])
            y0 = _atof(argv[3])
            z0 = _atof(argv[4])
            if self.polar:
                r, th, ph = x0, y0 * M_PI / 180.0, z0 * M_PI / 180.0
                x0 = r * math.sin(ph) * math.cos(th)
                y0 = r * math.sin(ph) * math.sin(th)
                z0 = r * math.cos(ph)
            else:
                y0 *= 1.0e-6
                z0 *= 1.0e-6
        x = 1.0e-6 * _atof(argv[off + 2])
        y = _atof(argv[off + 3])
        z = _atof(argv[off + 4])
        if self.polar:
            r, th, ph = x, y * M_PI / 180.0, z * M_PI / 180.0
            x = r * math.sin(ph) * math.cos(th)
            y = r * math.sin(ph) * math.sin(th)
            z = r * math.cos(ph)
        else:
            y *= 1.0e-6
            z *= 1.0e-6
        d = 1.0e-6 * _atof(argv[off + 5])
        c = self._compartment(argv[0], argv[1], x0, y0, z0, x, y, z, d)
        if c is not None:
            self._channels(c, argv)

    # ---- buildCompartment
    def _compartment(self, name, parent, x0, y0, z0, x, y, z, d):
        if parent == ".":
            pa = self.last
        elif parent in ("none", "nil"):
            pa = None
        else:
            pa = self.by_name.get(parent)
            if pa is None:
                self._warn("could not find parent compt '%s' for child '%s'" % (parent, name))
                return None
        if name in self.by_name:
            raise ValueError("line %d: a second compartment named %s" % (self.line_num, name))
        c = _Compt()
        c.name, c.parent, c.objs, c.inject = name, pa, [], 0.0
        c.sym, c.distal, c.sibs = bool(self.symmetric), [], []
        if self.proto is not None:
            if self.proto.symmetric != c.sym:
                raise ValueError("line %d: a %s prototype under %s" % (
                    self.line_num, "SymCompartment" if self.proto.symmetric else "Compartment",
                    "*symmetric" if c.sym else "*asymmetric"))
            # Shell::doCopy: the children with their values, their messages
            c.objs = [[n, p, dict(f)] for n, p, f in self.proto.children]
            for src, sf, dst, df in self.proto.msgs:
                self._link(c, src, sf, dst, df, "%s %s %s %s" % (src, sf, dst, df))
            c.inject = self.proto.inject
        if pa is not None and c.sym and not self.compts[pa].sym:
            raise ValueError("line %d: symmetric compartment %s on the non-symmetric parent %s (ReadCell's "
                             "distal -> proximal message needs a SymCompartment at both ends)"
                             % (self.line_num, name, self.compts[pa].name))
        idx = len(self.compts)
        self.compts.append(c)
        self.by_name[name] = idx
        self.last = idx
        if pa is not None:
            p = self.compts[pa]
            px, py, pz = p.x, p.y, p.z
            if not self.double_endpoint:
                x0, y0, z0 = px, py, pz
            if self.relative == 1:
                x += px
                y += py
                z += pz
                if self.double_endpoint:
                    x0 += px
                    y0 += py
                    z0 += pz
            dx, dy, dz = x - x0, y - y0, z - z0
            length = math.sqrt(dx * dx + dy * dy + dz * dz)
            if c.sym:
                # ReadCell: the parent's distalOut targets before this child
                # (its children and its siblings) become siblings, then the
                # distal -> proximal message, then the sibling messages
                # (both ends send distalOut)
                c.sibs = list(p.distal)
                p.distal.append(idx)
                for q in c.sibs:
                    c.distal.append(q)
                    self.compts[q].distal.append(idx)
        else:
            length = math.sqrt(x * x + y * y + z * z)
        surf = calc_surf(length, d)
        c.Cm = self.CM * surf
        c.Rm = self.RM / surf
        c.Ra = self.RA * length * 4.0 / (d * d * M_PI) if length > 0 else self.RA * 8.0 / (d * M_PI)
        eleak = self.EREST_ACT if (self.erest_flag and not self.eleak_flag) else self.ELEAK
        erest = self.ELEAK if (not self.erest_flag and self.eleak_flag) else self.EREST_ACT
        # CompartmentBase setters in the order ReadCell calls them: the
        # coordinates (each recomputing length_), then setLength, which
        # rescales the end point when length_ agrees with the coordinates
        cur = math.sqrt((x - x0) * (x - x0) + (y - y0) * (y - y0) + (z - z0) * (z - z0))
        if length > 0 and cur > 0 and _double_eq(cur * cur, (x - x0) * (x - x0) + (y - y0) * (y - y0)
                                                 + (z - z0) * (z - z0)):
            ratio = length / cur
            x = x0 + ratio * (x - x0)
            y = y0 + ratio * (y - y0)
            z = z0 + ratio * (z - z0)
        c.x0, c.y0, c.z0, c.x, c.y, c.z, c.d, c.length = x0, y0, z0, x, y, z, d, length
        c.initVm, c.Em = erest, eleak
        return c

    # ---- buildChannels
    def _channels(self, c, argv):
        if self.double_endpoint:
            ok, start = len(argv) % 2 == 1, 9
        else:
            ok, start = len(argv) % 2 == 0, 6
        if not ok:
            self._warn("bad number of arguments in channel list")
            return
        good = []
        j = start
        while j < len(argv):
            chan = argv[j]
            j += 1
            value = _atof(argv[j])
            if chan == "RA":
                c.Ra = (8.0 * value / (c.d * M_PI) if c.length == 0.0
                        else 4.0 * value * c.length / (c.d * c.d * M_PI))
            elif chan == "RM":
                c.Rm = value * calc_surf(c.length, c.d)
            elif chan == "CM":
                c.Cm = value * calc_surf(c.length, c.d)
            elif chan == "Rm":
                c.Rm = value
            elif chan == "Ra":
                c.Ra = value
            elif chan == "Cm":
                c.Cm = value
            elif chan == "kinModel":
                if j + 2 < len(argv):
                    j += 2
                else:
                    self._warn("kinModel needs 3 args")
                    break
            elif chan in ("m2c", "c2m"):
                if j + 4 < len(argv):
                    j += 4
                else:
                    self._warn("%s adaptor needs 5 args" % chan)
                    break
            else:
                proto = self.lib.get(chan)
                if proto is None:
                    self._warn("channel '%s' not found" % chan)
                elif any(o[0] == chan for o in c.objs):
                    raise ValueError("line %d: %s twice in compartment %s" % (self.line_num, chan, c.name))
                else:
                    o = self._add(c, chan, proto, value)
                    if o is not None:
                        good.append(o)
            j += 1
        for o in good:
            self._wire(c, o)

    def _add(self, c, name, proto, value):
        if isinstance(proto, (HHChannelProto, HHChannel2DProto, SynChanProto)):
            g = value * calc_surf(c.length, c.d) if value > 0 else -value
            o = [name, proto, {"Gbar": g}]
        elif isinstance(proto, SpikeGenProto):
            o = [name, proto, {"threshold": value}]
        elif isinstance(proto, CaConcProto):
            t = proto.thick if proto.thick <= c.d / 2.0 else 0.0
            if value > 0.0:
                if c.length > 0.0:
                    vol = M_PI * c.length * (c.d - t) * t if t > 0.0 else c.d * c.d * M_PI * c.length / 4.0
                else:
                    inner = c.d - 2 * t
                    vol = (M_PI * (c.d * c.d * c.d - inner * inner * inner) / 6.0 if t > 0.0
                           else M_PI * c.d * c.d * c.d / 6.0)
                if vol > 0.0:
                    value /= vol
            else:
                value = -value
            o = [name, proto, {"B_readcell": value}]
        else:
            self._warn("object '%s' is not a channel, CaConc or SpikeGen" % name)
            return None
        c.objs.append(o)
        return o

    def _wire(self, c, o):
        """addChannelMessage: the prototype's addmsg strings."""
        here = {x[0]: x for x in c.objs}

        def find(path):
            if path == ".":
                return o
            if path.startswith("../") and path[3:] in here:
                return here[path[3:]]
            return None

        for s in o[1].addmsg:
            t = _tokens(s)
            if len(t) != 4:
                raise ValueError("addmsg '%s': four fields expected" % s)
            src, dst = find(t[0]), find(t[2])
            if src is None or dst is None:
                continue             # as the reference: a missing end skips the message
            self._link(c, src[0], t[1], dst[0], t[3], s)

    def _link(self, c, src_name, sf, dst_name, df, text):
        """A message between two objects of compartment `c`."""
        here = {x[0]: x for x in c.objs}
        src, dst = here.get(src_name), here.get(dst_name)
        if src is None or dst is None:
            raise ValueError("message '%s': no object %s" % (text, src_name if src is None else dst_name))
        if sf == "IkOut" and df == "current" and isinstance(src[1], HHChannelProto) \
                and isinstance(dst[1], CaConcProto):
            src[2]["ca_target"] = dst[0]
        elif sf == "concOut" and df in ("concen", "concen2") and isinstance(src[1], CaConcProto) \
                and isinstance(dst[1], (HHChannelProto, HHChannel2DProto)):
            key = "ca_depend" if isinstance(dst[1], HHChannelProto) else ("conc1" if df == "concen" else "conc2")
            dst[2][key] = src[0]
        else:
            raise ValueError("addmsg '%s' is not supported" % text)


def read_cell(path, library):
    """Parse a .p file with the given channel library (``ReadCell::read``)."""
    with open(path, "r", encoding="latin-1") as f:
        return ReadCell(library).read(f.read())


def load_p(path, library, seed=0):
    """A .p file as a ``CellModel`` (tree walk from compartment `seed`, the
    HSolve target; by default the first compartment of the file)."""
    rc = read_cell(path, library)
    cs = rc.compts
    n = len(cs)
    if n == 0:
        raise ValueError("%s: no compartments" % path)
    gates, gate_ix = [], {}
    gates2d, gate2d_ix = [], {}

    def gate(pname, letter, g):
        k = (pname, letter)
        if k not in gate_ix:
            gate_ix[k] = len(gates)
            gates.append((float(g[0]), float(g[1]), np.asarray(g[2], float), np.asarray(g[3], float)))
        return gate_ix[k]

    ch = {k: [] for k in ("compt", "Gbar", "Ek", "Xp", "Yp", "Zp", "xg", "yg", "zg", "inst", "conc", "tgt", "dep")}
    c2 = {k: [] for k in ("compt", "Gbar", "Ek", "Xp", "xg", "xi", "c1", "c2")}
    pool = {k: [] for k in ("compt", "Ca", "basal", "tau", "B", "ceil", "floor", "d", "L", "thick")}
    sg = {k: [] for k in ("compt", "th", "ref", "edge")}
    sy = {k: [] for k in ("compt", "Gbar", "Ek", "tau1", "tau2", "name")}
    pool_of = []              # per compartment: CaConc name -> pool index
    for i, c in enumerate(cs):
        names = {}
        for name, proto, f in c.objs:
            if isinstance(proto, CaConcProto):
                names[name] = len(pool["compt"])
                pool["compt"].append(i)
                pool["Ca"].append(proto.CaBasal)
                pool["basal"].append(proto.CaBasal)
                pool["tau"].append(proto.tau)
                pool["B"].append(proto.zombie_B())
                pool["ceil"].append(proto.ceiling)
                pool["floor"].append(proto.floor)
                pool["d"].append(proto.diameter)
                pool["L"].append(proto.length)
                pool["thick"].append(proto.thick)
        pool_of.append(names)
    for i, c in enumerate(cs):
        for name, proto, f in c.objs:
            if isinstance(proto, HHChannelProto):
                ch["compt"].append(i)
                ch["Gbar"].append(f["Gbar"])
                ch["Ek"].append(proto.Ek)
                ch["Xp"].append(proto.Xpower)
                ch["Yp"].append(proto.Ypower)
                ch["Zp"].append(proto.Zpower)
                ch["xg"].append(gate(name, "X", proto.xgate) if proto.Xpower > 0 else -1)
                ch["yg"].append(gate(name, "Y", proto.ygate) if proto.Ypower > 0 else -1)
                ch["zg"].append(gate(name, "Z", proto.zgate) if proto.Zpower > 0 else -1)
                ch["inst"].append(proto.instant)
                ch["conc"].append(proto.useConcentration)
                ch["tgt"].append(pool_of[i][f["ca_target"]] if "ca_target" in f else -1)
                ch["dep"].append(pool_of[i][f["ca_depend"]] if "ca_depend" in f else -1)
            elif isinstance(proto, HHChannel2DProto):
                if name not in gate2d_ix:
                    gate2d_ix[name] = len(gates2d)
                    xmn, xmx, ymn, ymx, A, B = proto.table
                    gates2d.append((float(xmn), float(xmx), float(ymn), float(ymx), np.asarray(A, float),
                                    np.asarray(B, float)))
                c2["compt"].append(i)
                c2["Gbar"].append(f["Gbar"])
                c2["Ek"].append(proto.Ek)
                c2["Xp"].append(proto.Xpower)
                c2["xg"].append(gate2d_ix[name])
                c2["xi"].append(HS_DEP[proto.Xindex])
                c2["c1"].append(pool_of[i][f["conc1"]] if "conc1" in f else -1)
                c2["c2"].append(pool_of[i][f["conc2"]] if "conc2" in f else -1)
            elif isinstance(proto, SpikeGenProto):
                sg["compt"].append(i)
                sg["th"].append(f["threshold"])
                sg["ref"].append(proto.refractT)
                sg["edge"].append(proto.edgeTriggered)
            elif isinstance(proto, SynChanProto):
                sy["compt"].append(i)
                sy["Gbar"].append(f["Gbar"])
                sy["Ek"].append(proto.Ek)
                sy["tau1"].append(proto.tau1)
                sy["tau2"].append(proto.tau2)
                sy["name"].append(name)
    nc, n2 = len(ch["compt"]), len(c2["compt"])
    f64 = lambda v: np.asarray(v, np.float64)
    i32 = lambda v: np.asarray(v, np.int32)
    u32 = lambda v: np.asarray(v, np.uint32)
    m = CellModel(
        seed=seed, gates=gates, gates2d=gates2d,
        parent=i32([-1 if c.parent is None else c.parent for c in cs]),
        Ra=f64([c.Ra for c in cs]), Rm=f64([c.Rm for c in cs]), Cm=f64([c.Cm for c in cs]),
        Em=f64([c.Em for c in cs]), initVm=f64([c.initVm for c in cs]), Vm=f64([c.initVm for c in cs]),
        inject=f64([c.inject for c in cs]),
        chan_compt=u32(ch["compt"]), chan_Gbar=f64(ch["Gbar"]), chan_Ek=f64(ch["Ek"]),
        chan_Xpower=f64(ch["Xp"]), chan_Ypower=f64(ch["Yp"]), chan_Zpower=f64(ch["Zp"]),
        chan_xgate=i32(ch["xg"]), chan_ygate=i32(ch["yg"]), chan_zgate=i32(ch["zg"]),
        chan_instant=i32(ch["inst"]), chan_modulation=np.ones(nc), chan_use_conc=i32(ch["conc"]),
        chan_X=np.zeros(nc), chan_Y=np.zeros(nc), chan_Z=np.zeros(nc),
        chan_ca_target=i32(ch["tgt"]), chan_ca_depend=i32(ch["dep"]),
        pool_compt=u32(pool["compt"]), pool_Ca=f64(pool["Ca"]), pool_CaBasal=f64(pool["basal"]),
        pool_tau=f64(pool["tau"]), pool_B=f64(pool["B"]), pool_ceiling=f64(pool["ceil"]),
        pool_floor=f64(pool["floor"]),
        c2d_compt=u32(c2["compt"]), c2d_Gbar=f64(c2["Gbar"]), c2d_Ek=f64(c2["Ek"]), c2d_Xpower=f64(c2["Xp"]),
        c2d_xgate=i32(c2["xg"]), c2d_xindex=i32(c2["xi"]), c2d_conc1_pool=i32(c2["c1"]),
        c2d_conc2_pool=i32(c2["c2"]), c2d_instant=np.zeros(n2, np.int32), c2d_modulation=np.ones(n2),
        c2d_X=np.zeros(n2),
        sg_compt=u32(sg["compt"]), sg_threshold=f64(sg["th"]), sg_refractT=f64(sg["ref"]),
        sg_edge=i32(sg["edge"]),
        syn_compt=u32(sy["compt"]), syn_Gbar=f64(sy["Gbar"]), syn_Ek=f64(sy["Ek"]), syn_tau1=f64(sy["tau1"]),
        syn_tau2=f64(sy["tau2"]), syn_modulation=np.ones(len(sy["compt"])),
        ev_syn=np.zeros(0, np.uint32), ev_time=np.zeros(0), ev_weight=np.zeros(0),
        meta={"names": [c.name for c in cs], "diameter": f64([c.d for c in cs]),
              "length": f64([c.length for c in cs]),
              "coords": f64([(c.x0, c.y0, c.z0, c.x, c.y, c.z) for c in cs]).reshape(-1, 6),
              "chan_name": [o[0] for c in cs for o in c.objs if isinstance(o[1], HHChannelProto)],
              "syn_name": sy["name"],
              "syn_weight": f64([o[1].weight for c in cs for o in c.objs if isinstance(o[1], SynChanProto)]),
              "pool_diameter": f64(pool["d"]), "pool_length": f64(pool["L"]), "pool_thick": f64(pool["thick"]),
              "classes": ["SymCompartment" if c.sym else "Compartment" for c in cs],
              "sibling_links": [(i, q) for i, c in enumerate(cs) for q in c.sibs],
              "warnings": rc.warnings})
    return m
