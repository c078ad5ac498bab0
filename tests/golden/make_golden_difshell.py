#!/usr/bin/env python3
"""External-calcium golden from the reference's own test.

Runs the reference's `tests/core/test_hsolve_externalCalcium.py`
(`test_hsolve_calcium`, unmodified, from the reference tree) with the
reference build's pymoose: a GENESIS soma with a CaL12 channel whose IkOut
feeds the outer of three DifShells (`influx`) and an SK channel whose Z
gate reads that shell's concentration (`concentrationOut -> concen`, i.e.
HSolve::addConc), under HSolve at dt = 10 us for 10 s (1,000,000 steps),
Tables every 5 ms.  The test's own assertions run and must pass.

Just before the test's `moose.reinit()`, the MOOSE-side binding
(`hsb_fill_cell_desc`, moose-core_gb300/cpp/moose_hsolve_bridge.cpp, linked
into the reference build) describes the set-up solver, the three DifShells
and their messages included; that description is saved as the model.
Saved: the soma Vm, the outer shell's C, the SK and CaL12 conductances
(2,001 samples each), the indices of the recorded objects in the
description, and the test's expected statistics (read from the test file).

Prerequisite: the reference build (python oracle/build_ref.py).
"""
import ast
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
from build_ref import source_dir  # noqa: E402
REF_CORE = os.path.join(source_dir(), "tests", "core")
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
sys.path.insert(0, os.path.join(REPO, "moose-core_gb300"))

from loader import model_from_desc  # noqa: E402
from make_golden_active import save_model  # noqa: E402
from moose_gb300.abi import HsCellDesc  # noqa: E402


def expected_stats():
    """The two assert_stat expectations of the test, read as literals."""
    tree = ast.parse(open(os.path.join(REF_CORE, "test_hsolve_externalCalcium.py")).read())
    out = []
    for node in ast.walk(tree):
        if isinstance(node, ast.Call) and getattr(node.func, "id", None) == "assert_stat":
            out.append(ast.literal_eval(node.args[1]))
    return out


def main():
    import moose
    sys.path.insert(0, REF_CORE)
    os.chdir(REF_CORE)          # the test's helpers read files next to it
    import test_hsolve_externalCalcium as T
    L = C.CDLL(moose._moose.__file__)
    L.hsb_fill_cell_desc.restype = C.POINTER(HsCellDesc)
    L.hsb_fill_cell_desc.argtypes = [C.c_char_p, C.POINTER(C.c_uint32)]
    L.hsb_free_cell_desc.argtypes = [C.POINTER(HsCellDesc)]
    L.hsb_object_path.argtypes = [C.POINTER(HsCellDesc), C.c_int, C.c_uint32, C.c_char_p, C.c_uint32]
    L.hsb_last_error.restype = C.c_char_p
    captured = {}
    real_reinit = moose.reinit

    def reinit_with_capture(*a, **k):
        seed = C.c_uint32()
        d = L.hsb_fill_cell_desc(b"/neuron/hsolve", C.byref(seed))
        assert d, L.hsb_last_error()
        captured["model"] = model_from_desc(d.contents, seed.value)
        buf = C.create_string_buffer(512)
        paths = {}
        for kind, n in ((1, d.contents.n_chan), (6, d.contents.n_dif)):
            out = []
            for i in range(n):
                assert L.hsb_object_path(d, kind, i, buf, 512) >= 0
                out.append(buf.value.decode())
            paths[kind] = out
        captured["paths"] = paths
        L.hsb_free_cell_desc(d)
        return real_reinit(*a, **k)

    moose.reinit = reinit_with_capture
    try:
        T.test_hsolve_calcium()        # builds, runs 10 s, asserts its known answers
    finally:
        moose.reinit = real_reinit
    m = captured["model"]
    chans, difs = captured["paths"][1], captured["paths"][6]
    sk = next(i for i, p in enumerate(chans) if p.endswith("/SK"))
    cal = next(i for i, p in enumerate(chans) if p.endswith("/CaL12"))
    shell0 = next(i for i, p in enumerate(difs) if p.rstrip("]").split("/")[-1].startswith("Ca_shell0"))
    vm = np.array(moose.element("/data/Vm").vector)
    ca = np.array(moose.element("/data/Ca").vector)
    skg = np.array(moose.element("/data/SK_Gk").vector)
    calg = np.array(moose.element("/data/CaL_Gk").vector)
    kat_sk, kat_ca = expected_stats()
    print("model: %d compartments, %d channels, %d tick-1 objects, %d messages"
          % (m.n_compt, len(m.chan_compt), len(m.dif_kind), len(m.dmsg_kind)))
    print("samples", len(vm), "shell0", difs[shell0], "SK", chans[sk])
    np.savez_compressed(os.path.join(HERE, "ext_calcium.npz"),
                        dt=1e-5, nsteps=1000000, stride=500, vm=vm, shell_c=ca, sk_gk=skg, cal_gk=calg,
                        shell_index=shell0, sk_index=sk, cal_index=cal,
                        kat_sk=np.array(kat_sk), kat_ca=np.array(kat_ca),
                        **save_model(m))


if __name__ == "__main__":
    main()
