"""ctypes mirror of ``include/moose_gb300.h`` and the ``CellModel`` container.

``CellModel`` holds one cell as numpy arrays in the layout of ``HsCellDesc``
(what ``HSolveActive::setup`` reads from MOOSE objects,
``hsolve/HSolveActiveSetup.cpp:17-41``).  ``CellModel.desc()`` returns the C
struct pointing into those arrays; the model must outlive every use of it.
"""
import ctypes as C

import numpy as np

HS_OK, HS_EINVAL, HS_EDEVICE, HS_ENOMEM, HS_ETIMEOUT, HS_ESTATE, HS_ENOTSUP, HS_ECAPACITY = range(8)
HS_PREC_FP64, HS_PREC_MIXED = 0, 1

HS_DEP = {"VOLT_INDEX": 0, "C1_INDEX": 1, "C2_INDEX": 2, "VOLT_C1_INDEX": 3,
          "VOLT_C2_INDEX": 4, "C1_C2_INDEX": 5}

HS_KIND_COMPT, HS_KIND_CHAN, HS_KIND_POOL, HS_KIND_CHAN2D, HS_KIND_SYNCHAN = range(5)
FIELDS = {
    "Vm": 0, "Cm": 1, "Em": 2, "Rm": 3, "Ra": 4, "initVm": 5, "Im": 6, "inject": 7,
    "Gbar": 10, "Ek": 11, "Gk": 12, "Ik": 13, "X": 14, "Y": 15, "Z": 16,
    "instant": 17, "modulation": 18, "Xpower": 19, "Ypower": 20, "Zpower": 21,
    "Ca": 30, "CaBasal": 31, "ceiling": 32, "floor": 33, "tau": 34, "B": 35,
}

_pd = C.POINTER(C.c_double)
_pi = C.POINTER(C.c_int32)
_pu = C.POINTER(C.c_uint32)


class HsGateTable(C.Structure):
    _fields_ = [("min", C.c_double), ("max", C.c_double), ("divs", C.c_uint32),
                ("A", _pd), ("B", _pd)]


class HsGate2DTable(C.Structure):
    _fields_ = [("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double),
                ("ymax", C.c_double), ("xdivs", C.c_uint32), ("ydivs", C.c_uint32),
                ("A", _pd), ("B", _pd)]


# (field name, ctypes pointer type or scalar type) in header order.
_DESC_FIELDS = [
    ("n_compt", C.c_uint32), ("parent", _pi), ("Ra", _pd), ("Rm", _pd), ("Cm", _pd),
    ("Em", _pd), ("initVm", _pd), ("Vm", _pd), ("inject", _pd),
    ("n_leak", C.c_uint32), ("leak_compt", _pu), ("leak_Ek", _pd), ("leak_Gk", _pd),
    ("n_gate", C.c_uint32), ("gate", C.POINTER(HsGateTable)),
    ("n_chan", C.c_uint32), ("chan_compt", _pu), ("chan_Gbar", _pd), ("chan_Ek", _pd),
    ("chan_Xpower", _pd), ("chan_Ypower", _pd), ("chan_Zpower", _pd),
    ("chan_xgate", _pi), ("chan_ygate", _pi), ("chan_zgate", _pi), ("chan_instant", _pi),
    ("chan_modulation", _pd), ("chan_use_conc", _pi), ("chan_X", _pd), ("chan_Y", _pd),
    ("chan_Z", _pd), ("chan_ca_target", _pi), ("chan_ca_depend", _pi),
    ("n_pool", C.c_uint32), ("pool_compt", _pu), ("pool_Ca", _pd), ("pool_CaBasal", _pd),
    ("pool_tau", _pd), ("pool_B", _pd), ("pool_ceiling", _pd), ("pool_floor", _pd),
    ("n_gate2d", C.c_uint32), ("gate2d", C.POINTER(HsGate2DTable)),
    ("n_chan2d", C.c_uint32), ("c2d_compt", _pu), ("c2d_Gbar", _pd), ("c2d_Ek", _pd),
    ("c2d_Xpower", _pd), ("c2d_xgate", _pi), ("c2d_xindex", _pi), ("c2d_conc1_pool", _pi),
    ("c2d_conc2_pool", _pi), ("c2d_instant", _pi), ("c2d_modulation", _pd), ("c2d_X", _pd),
    ("n_syn", C.c_uint32), ("syn_compt", _pu), ("syn_Gbar", _pd), ("syn_Ek", _pd),
    ("syn_tau1", _pd), ("syn_tau2", _pd), ("syn_modulation", _pd),
    ("n_event", C.c_uint32), ("ev_syn", _pu), ("ev_time", _pd), ("ev_weight", _pd),
    ("n_spikegen", C.c_uint32), ("sg_compt", _pu), ("sg_threshold", _pd),
    ("sg_refractT", _pd), ("sg_edge", _pi),
    ("n_stim", C.c_uint32), ("stim_compt", _pu), ("stim_step", _pu), ("stim_value", _pd),
    ("n_dif", C.c_uint32), ("dif_kind", _pi), ("difpar", _pd),
    ("n_dmsg", C.c_uint32), ("dmsg_kind", _pi), ("dmsg_src", _pu), ("dmsg_dst", _pu),
    ("link", _pi),
]

# how a compartment hangs on its parent (include/moose_gb300.h HS_LINK_*)
HS_LINK_AXIAL, HS_LINK_DISTAL, HS_LINK_CYLINDER = 0, 1, 2

# tick-1 external calcium objects (include/moose_gb300.h HS_DIF_*, HS_DMSG_*)
HS_DIF_SHELL, HS_DIF_BUFFER, HS_DIF_PUMP = 0, 1, 2
HS_DIF_NPAR = 12
(HS_DMSG_OUTER, HS_DMSG_INNER, HS_DMSG_CONC_CHAN, HS_DMSG_CONC_BUF, HS_DMSG_REACTION, HS_DMSG_PUMP,
 HS_DMSG_IK) = range(7)


class HsCellDesc(C.Structure):
    _fields_ = _DESC_FIELDS


class HsBatchTuning(C.Structure):
    _fields_ = [("threads_per_cta", C.c_uint32), ("ctas_per_sm", C.c_uint32),
                ("steps_per_launch", C.c_uint32), ("use_graph", C.c_uint32),
                ("forest_nodes", C.c_uint32), ("max_ctas", C.c_uint32), ("elim_warps", C.c_uint32),
                ("wait_rounds", C.c_uint32), ("cluster_ctas", C.c_uint32)]


# numpy dtype per array field
_F64 = np.float64
_I32 = np.int32
_U32 = np.uint32
_ARRAYS = {
    "parent": _I32, "Ra": _F64, "Rm": _F64, "Cm": _F64, "Em": _F64, "initVm": _F64,
    "Vm": _F64, "inject": _F64,
    "leak_compt": _U32, "leak_Ek": _F64, "leak_Gk": _F64,
    "chan_compt": _U32, "chan_Gbar": _F64, "chan_Ek": _F64, "chan_Xpower": _F64,
    "chan_Ypower": _F64, "chan_Zpower": _F64, "chan_xgate": _I32, "chan_ygate": _I32,
    "chan_zgate": _I32, "chan_instant": _I32, "chan_modulation": _F64, "chan_use_conc": _I32,
    "chan_X": _F64, "chan_Y": _F64, "chan_Z": _F64, "chan_ca_target": _I32,
    "chan_ca_depend": _I32,
    "pool_compt": _U32, "pool_Ca": _F64, "pool_CaBasal": _F64, "pool_tau": _F64,
    "pool_B": _F64, "pool_ceiling": _F64, "pool_floor": _F64,
    "c2d_compt": _U32, "c2d_Gbar": _F64, "c2d_Ek": _F64, "c2d_Xpower": _F64,
    "c2d_xgate": _I32, "c2d_xindex": _I32, "c2d_conc1_pool": _I32, "c2d_conc2_pool": _I32,
    "c2d_instant": _I32, "c2d_modulation": _F64, "c2d_X": _F64,
    "syn_compt": _U32, "syn_Gbar": _F64, "syn_Ek": _F64, "syn_tau1": _F64, "syn_tau2": _F64,
    "syn_modulation": _F64,
    "ev_syn": _U32, "ev_time": _F64, "ev_weight": _F64,
    "sg_compt": _U32, "sg_threshold": _F64, "sg_refractT": _F64, "sg_edge": _I32,
    "stim_compt": _U32, "stim_step": _U32, "stim_value": _F64,
    "dif_kind": _I32, "difpar": _F64,
    "dmsg_kind": _I32, "dmsg_src": _U32, "dmsg_dst": _U32,
    "link": _I32,
}
# per-compartment arrays that may be left empty (NULL in the description)
_OPTIONAL = {"link"}
_COUNTS = {
    "n_compt": "parent", "n_leak": "leak_compt", "n_chan": "chan_compt",
    "n_pool": "pool_compt", "n_chan2d": "c2d_compt", "n_syn": "syn_compt",
    "n_event": "ev_syn", "n_spikegen": "sg_compt", "n_stim": "stim_compt",
    "n_dif": "dif_kind", "n_dmsg": "dmsg_kind",
}


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class CellModel:
    """One cell as SoA numpy arrays, in ``HsCellDesc`` layout.

    Gate tables: ``gates`` is a list of (min, max, A, B) with len(A) = divs+1;
    ``gates2d`` a list of (xmin, xmax, ymin, ymax, A[x][y], B[x][y]).
    ``seed`` is the compartment HSolve starts its tree walk from (the one
    found under ``HSolve.target``).
    """

    def __init__(self, **arrays):
        self.seed = int(arrays.pop("seed", 0))
        self.gates = arrays.pop("gates", [])
        self.gates2d = arrays.pop("gates2d", [])
        # Python-side metadata that is not part of HsCellDesc (e.g. pool geometry)
        self.meta = dict(arrays.pop("meta", {}) or {})
        for name, dt in _ARRAYS.items():
            v = arrays.pop(name, None)
            v = np.zeros(0, dt) if v is None else np.ascontiguousarray(v, dtype=dt)
            setattr(self, name, v)
        if arrays:
            raise TypeError("unknown CellModel fields: %s" % sorted(arrays))
        self._keep = None

    @property
    def n_compt(self):
        return len(self.parent)

    def validate(self):
        groups = {"parent": ("Ra", "Rm", "Cm", "Em", "initVm", "Vm", "inject", "link")}
        for first in _COUNTS.values():
            if first != "parent":
                prefix = first.split("_")[0] + "_"
                groups[first] = tuple(k for k in _ARRAYS if k.startswith(prefix))
        for first, members in groups.items():
            n = len(getattr(self, first))
            for name in members:
                if name in _OPTIONAL and len(getattr(self, name)) == 0:
                    continue
                if len(getattr(self, name)) != n:
                    raise ValueError("array %s has length %d, expected %d"
                                     % (name, len(getattr(self, name)), n))
        if len(self.difpar) != HS_DIF_NPAR * len(self.dif_kind):
            raise ValueError("difpar has length %d, expected %d" % (len(self.difpar),
                                                                    HS_DIF_NPAR * len(self.dif_kind)))

    def desc(self):
        """Build an ``HsCellDesc`` pointing into this model's arrays.

        A model whose SymCompartments are joined by sibling messages (a
        GENESIS ``*symmetric`` cell with a branch point, ``meta["sibling_links"]``)
        is refused: the reference HSolve's tree walk follows the sibling
        messages' ``distalOut`` (``hsolve/HSolveUtils.cpp:36-45``) and never
        ends, so there is no reference setup to reproduce."""
        links = self.meta.get("sibling_links")
        if links is not None and len(links):
            raise ValueError("SymCompartments joined by sibling messages (%d links, e.g. compartments %d and %d): "
                             "the reference HSolve cannot set this cell up (its tree walk follows them)"
                             % (len(links), links[0][0], links[0][1]))
        self.validate()
        d = HsCellDesc()
        keep = []
        for name, dt in _ARRAYS.items():
            a = getattr(self, name)
            ct = {np.float64: C.c_double, np.int32: C.c_int32, np.uint32: C.c_uint32}[np.dtype(dt).type]
            setattr(d, name, _ptr(a, ct) if len(a) else None)
        for cnt, first in _COUNTS.items():
            setattr(d, cnt, len(getattr(self, first)))
        gt = (HsGateTable * max(1, len(self.gates)))()
        for i, (mn, mx, A, B) in enumerate(self.gates):
            A = np.ascontiguousarray(A, np.float64)
            B = np.ascontiguousarray(B, np.float64)
            if len(A) != len(B) or len(A) < 2:
                raise ValueError("gate %d: tableA/tableB must have equal length >= 2" % i)
            keep += [A, B]
            gt[i] = HsGateTable(float(mn), float(mx), len(A) - 1, _ptr(A, C.c_double), _ptr(B, C.c_double))
        d.n_gate = len(self.gates)
        d.gate = gt
        g2 = (HsGate2DTable * max(1, len(self.gates2d)))()
        for i, (xmn, xmx, ymn, ymx, A, B) in enumerate(self.gates2d):
            A = np.ascontiguousarray(A, np.float64)
            B = np.ascontiguousarray(B, np.float64)
            if A.shape != B.shape or A.ndim != 2:
                raise ValueError("gate2d %d: A and B must be equal 2-D arrays" % i)
            keep += [A, B]
            g2[i] = HsGate2DTable(float(xmn), float(xmx), float(ymn), float(ymx),
                                  A.shape[0] - 1, A.shape[1] - 1,
                                  _ptr(A, C.c_double), _ptr(B, C.c_double))
        d.n_gate2d = len(self.gates2d)
        d.gate2d = g2
        self._keep = (keep, gt, g2, d)
        return d

    def total_states(self):
        return int((self.chan_Xpower > 0).sum() + (self.chan_Ypower > 0).sum() + (self.chan_Zpower > 0).sum())
