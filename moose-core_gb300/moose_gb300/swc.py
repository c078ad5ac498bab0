"""SWC morphology reader: compartmental cells for the solver from NeuroMorpho
SWC files, built the way MOOSE's ``loadModel`` builds them.

MOOSE reads an SWC file with ``ReadSwc`` (``biophysics/ReadSwc.cpp``) and
``SwcSegment`` (``biophysics/SwcSegment.cpp``), then ``ReadSwc::build`` makes
one Compartment per segment with RM = 1, RA = 1, CM = 0.01 as called from
``Shell::doLoadModel`` (``shell/LoadModels.cpp:155-165``).  This module does
the same steps, in the same order, so that a cell loaded here has the same
compartments, passive values (bit for bit), names, parent links and child
order as the reference's, and therefore the same Hines numbering once an
HSolve takes it over:

  * parsing (``SwcSegment::SwcSegment(const string&)``, ``SwcSegment.cpp:38-62``):
    a line of exactly seven whitespace-separated fields ``n type x y z r
    parent``; the integers are read like C ``atoi`` and the reals like
    ``atof`` (leading numeric prefix); parent <= 0 means none.  Lines that
    are empty, blank or start with ``#`` are skipped; lines with another
    field count, or of type 0 (undefined) or 7 (custom), count as bad and
    are dropped -- which shifts the positions of the lines after them, as in
    the reference, since parents are looked up by position;
  * validation (``ReadSwc::validate``, ``ReadSwc.cpp:70-113``): exactly one
    root, every parent earlier in the file, every radius >= 0.04 um.  An
    invalid file builds no compartments (the reference prints a message and
    builds nothing; ``load_swc`` raises);
  * children and segment types (``assignKids``, ``figureOutType``);
  * zero-length cleaning (``cleanZeroLength``, ``ReadSwc.cpp:131-160``): a
    segment closer than 0.01 um to its parent is dropped and its children
    move to the parent, after the parent's other children;
  * branches (``parseBranches``/``traverseBranch``, ``ReadSwc.cpp:162-215``):
    one branch per fork or end segment, running back up to the previous
    fork; branches in file order of their last segment;
  * compartments (``makeCompt``/``build``, ``ReadSwc.cpp:236-313``): branch
    after branch, segment after segment; length = distance to the parent
    segment (the soma: its diameter), Rm = RM/(len dia pi), Ra = RA len/xa
    with xa = r^2 pi 1e-12, Cm = CM (len dia pi), in metres; names ``soma``
    and ``<type>_<branch>_<segment>``.  Each compartment is joined to its
    parent as it is made, so a compartment's children are in creation order,
    which is index order here.
"""
import math
import re

import numpy as np

# constexpr PI of basecode/header.h
PI = 3.141592653589793
MIN_RADIUS = 0.04          # um (ReadSwc.cpp, MinRadius)
ZERO_LENGTH = 1e-2         # um (ReadSwc::cleanZeroLength, EPSILON)

UNDEF, SOMA, AXON, DEND, APICAL, FORK, END, CUSTOM, BAD = 0, 1, 2, 3, 4, 5, 6, 7, 8
AXON_FORK, AXON_END, APICAL_FORK, APICAL_END = 10, 11, 12, 13
TYPE_NAMES = ("undef", "soma", "axon", "dend", "apical", "dend_f", "dend_e", "custom", "bad", "undef",
              "axon_f", "axon_e", "apical_f", "apical_e")
NO_PARENT = 0xFFFFFFFF     # ~0U

_WS = re.compile(r"[ \t\n\v\f\r]+")   # what `istream >> string` skips
_INT = re.compile(r"\s*([+-]?\d+)")
_REAL = re.compile(r"\s*([+-]?(?:\d+\.?\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|inf(?:inity)?|nan))",
                   re.IGNORECASE)


def _atoi(s):
    """C atoi: the leading integer of `s`, 0 if there is none (32-bit wrap)."""
    m = _INT.match(s)
    if not m:
        return 0
    v = int(m.group(1))
    return ((v + 2 ** 31) % 2 ** 32) - 2 ** 31


def _atof(s):
    """C atof: the leading real number of `s`, 0.0 if there is none."""
    m = _REAL.match(s)
    return float(m.group(1)) if m else 0.0


class SwcSegment:
    """One SWC line (``SwcSegment``): 1-based index, type, position (um),
    radius (um), 1-based parent (NO_PARENT for the root), children."""

    __slots__ = ("index", "type", "x", "y", "z", "radius", "parent", "kids")

    def __init__(self, index, typ, x, y, z, radius, parent):
        self.index, self.type = index, typ
        self.x, self.y, self.z, self.radius = x, y, z, radius
        self.parent = parent
        self.kids = []

    @classmethod
    def parse(cls, line):
        args = [a for a in _WS.split(line) if a]
        if len(args) != 7:
            return cls(0, BAD, 0.0, 0.0, 0.0, 0.0, NO_PARENT)
        pa = _atoi(args[6])
        # myIndex_ is unsigned in the reference
        return cls(_atoi(args[0]) & 0xFFFFFFFF, _atoi(args[1]), _atof(args[2]), _atof(args[3]),
                   _atof(args[4]), _atof(args[5]), pa if pa > 0 else NO_PARENT)

    def ok(self):
        return self.type not in (BAD, UNDEF, CUSTOM)

    def distance(self, o):
        # Vec::distance: sqrt(a0 a0 + a1 a1 + a2 a2) of the difference
        a0, a1, a2 = self.x - o.x, self.y - o.y, self.z - o.z
        return math.sqrt(a0 * a0 + a1 * a1 + a2 * a2)

    def figure_out_type(self):
        n = len(self.kids)
        if self.type == DEND:
            self.type = FORK if n > 1 else END if n == 0 else DEND
        elif self.type == APICAL:
            self.type = APICAL_FORK if n > 1 else APICAL_END if n == 0 else APICAL
        elif self.type == AXON:
            self.type = AXON_FORK if n > 1 else AXON_END if n == 0 else AXON


class Swc:
    """A parsed SWC file: ``segs`` (in file order), ``bad`` (dropped lines),
    ``valid``, ``branches`` (lists of 1-based segment indices, root end
    first) and ``branch_parent``."""

    def __init__(self, text):
        self.segs = []
        self.bad = 0
        for line in text.split("\n"):       # getline: a '\r' stays in the line
            st = line.lstrip("\t ")
            if not st or st[0] == "#":
                continue
            s = SwcSegment.parse(line)
            if s.ok():
                self.segs.append(s)
            else:
                self.bad += 1
        self.branches, self.branch_parent = [], []
        self.valid = self._validate()
        if self.valid:
            self._assign_kids()
            self._clean_zero_length()
            self._parse_branches()

    def _validate(self):
        starts = orphans = small = 0
        for i, s in enumerate(self.segs):
            if s.parent == NO_PARENT:
                starts += 1
            elif s.parent > i:
                orphans += 1
            if s.radius < MIN_RADIUS:
                small += 1
        return starts == 1 and orphans == 0 and small == 0

    def _assign_kids(self):
        for i, s in enumerate(self.segs):
            if s.parent != NO_PARENT:
                self.segs[s.parent - 1].kids.append(i + 1)
        for s in self.segs:
            s.figure_out_type()

    def _clean_zero_length(self):
        for i in range(1, len(self.segs)):
            s = self.segs[i]
            pa = self.segs[s.parent - 1]
            if s.distance(pa) < ZERO_LENGTH:
                kept = [k for k in pa.kids if k != s.index]
                for k in s.kids:
                    kid = self.segs[k - 1]
                    kid.parent = pa.index
                    kept.append(kid.index)
                pa.kids = kept
                s.type = BAD

    def _traverse(self, s):
        """1-based segment indices from `s` up to (not including) the
        previous fork, nearest the root last (``traverseBranch``)."""
        cable = [s.index]
        if s.parent == NO_PARENT:
            return cable
        prev = s
        while True:
            pa = self.segs[prev.parent - 1]
            cable.append(pa.index)
            prev = pa
            if not (prev.parent != NO_PARENT and len(prev.kids) == 1):
                break
        cable.pop()
        return cable

    def _parse_branches(self):
        for s in self.segs:
            if s.ok() and len(s.kids) != 1:
                self.branches.append(self._traverse(s)[::-1])
        last = [0] * (len(self.segs) + 1)
        for i, br in enumerate(self.branches):
            last[br[-1]] = i
        for br in self.branches:
            pa = self.segs[br[0] - 1].parent
            self.branch_parent.append(last[pa] if pa != NO_PARENT else 0)


class SwcCompartments:
    """Compartments of a loaded SWC cell in creation order: ``names``,
    ``parent`` (index, -1 for the soma), ``Ra``, ``Rm``, ``Cm`` (ohm, ohm,
    F), ``diameter``, ``length`` (m; the end-to-end distance of the
    coordinates, as the Compartment reports it), ``elec_length`` (m; the
    distance between the SWC points, which the passive values use),
    ``x0 y0 z0 x y z`` (m), ``segment``
    (the 1-based SWC index of each)."""

    def __init__(self, **kw):
        self.__dict__.update(kw)

    def __len__(self):
        return len(self.names)


def build(swc, RM=1.0, RA=1.0, CM=0.01):
    """``ReadSwc::build``: one compartment per segment of each branch."""
    names, parent, seg_of = [], [], []
    Ra, Rm, Cm, dia, elec = [], [], [], [], []
    pos = []
    where = {}
    for i, br in enumerate(swc.branches):
        for j, k in enumerate(br):
            seg = swc.segs[k - 1]
            if seg.parent == NO_PARENT:
                pa = seg
                ln = seg.radius * 2.0
                name = "soma"
                x0, y0, z0 = seg.x - ln, seg.y, seg.z
                p = -1
            else:
                pa = swc.segs[seg.parent - 1]
                ln = seg.distance(pa)
                name = "%s_%d_%d" % (TYPE_NAMES[seg.type], i, j)
                x0, y0, z0 = pa.x, pa.y, pa.z
                if seg.parent not in where:
                    # e.g. a soma with exactly one child is not a branch end,
                    # so the reference makes no compartment for it either
                    raise ValueError("SWC segment %d: parent segment %d has no compartment" % (seg.index, seg.parent))
                p = where[seg.parent]
            xa = seg.radius * seg.radius * PI * 1e-12
            ln *= 1e-6
            d = seg.radius * 2.0e-6
            where[seg.index] = len(names)
            names.append(name)
            parent.append(p)
            seg_of.append(seg.index)
            Rm.append(RM / (ln * d * PI))
            Ra.append(RA * ln / xa)
            Cm.append(CM * (ln * d * PI))
            dia.append(d)
            elec.append(ln)
            pos.append((x0 * 1e-6, y0 * 1e-6, z0 * 1e-6, seg.x * 1e-6, seg.y * 1e-6, seg.z * 1e-6))
    pos = np.array(pos, dtype=np.float64).reshape(-1, 6)
    # the Compartment's length field ends as CompartmentBase::updateLength
    # computes it from the coordinates set last (CompartmentBase.cpp:508-512)
    length = [math.sqrt((x - x0) * (x - x0) + (y - y0) * (y - y0) + (z - z0) * (z - z0))
              for x0, y0, z0, x, y, z in pos.tolist()]
    return SwcCompartments(names=names, parent=np.array(parent, np.int32), Ra=np.array(Ra), Rm=np.array(Rm),
                           Cm=np.array(Cm), diameter=np.array(dia), length=np.array(length),
                           elec_length=np.array(elec),
                           x0=pos[:, 0], y0=pos[:, 1], z0=pos[:, 2], x=pos[:, 3], y=pos[:, 4], z=pos[:, 5],
                           segment=np.array(seg_of, np.int64))


def read_swc(path):
    """Parse an SWC file (``ReadSwc::ReadSwc``)."""
    with open(path, "r", encoding="latin-1", newline="") as f:
        return Swc(f.read())


def load_swc(path, RM=1.0, RA=1.0, CM=0.01, Em=-0.06, initVm=-0.06):
    """Compartments of an SWC file as ``loadModel`` builds them, as a passive
    ``CellModel`` whose tree walk starts at the soma.  Em and initVm default
    to MOOSE's Compartment defaults (-60 mV).  Raises ValueError for a file
    that fails validation."""
    from .abi import CellModel
    swc = read_swc(path)
    if not swc.valid:
        raise ValueError("SWC file %s failed validation (one root, parents before children, radius >= %g um)"
                         % (path, MIN_RADIUS))
    c = build(swc, RM, RA, CM)
    n = len(c)
    m = CellModel(seed=0, parent=c.parent, Ra=c.Ra, Rm=c.Rm, Cm=c.Cm, Em=np.full(n, Em),
                  initVm=np.full(n, initVm), Vm=np.full(n, initVm), inject=np.zeros(n))
    m.meta["names"] = c.names
    m.meta["diameter"] = c.diameter
    m.meta["length"] = c.length
    return m


def active_swc_cell(path, **kw):
    """An SWC morphology with the channels of ``models.active_cell`` (HH Na/K,
    Ca(HVA) into a CaConc, K(Ca) HHChannel2D; optional SynChans) on every
    compartment, with the passive values ``loadModel`` gives it.  Keyword
    arguments go to ``models.active_cell``."""
    from . import models
    swc = read_swc(path)
    if not swc.valid:
        raise ValueError("SWC file %s failed validation" % path)
    c = build(swc)
    area = c.elec_length * c.diameter * PI
    m = models.active_cell(c.parent, c.diameter, c.elec_length, passive_props=(c.Ra, c.Rm, c.Cm, area), **kw)
    m.meta["names"] = c.names
    return m
