"""The C-ABI library: it builds, loads, exports every function that
include/moose_gb300.h declares, and rejects bad models with status codes
(validation runs before any device work, so this needs no GPU)."""
import ctypes as C

import numpy as np
import pytest

from moose_gb300 import _native, models
from moose_gb300.abi import HS_EDEVICE, HS_EINVAL, HS_ENOTSUP, HS_PREC_FP64, HS_PREC_MIXED, CellModel


def test_library_exports_every_declared_symbol():
    L = _native.load()
    names = _native.declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_build_info():
    assert b"sm_103a" in _native.load().hs_build_info()


def _create(model, seed=0, dt=25e-6, prec=HS_PREC_FP64):
    L = _native.load()
    d = model.desc()
    h = C.c_void_p()
    rc = L.hs_create(C.byref(d), seed, dt, prec, C.byref(h))
    if rc == 0:
        L.hs_destroy(h)
    return rc, L.hs_last_error().decode()


def test_rejects_bad_models():
    m = models.config1_cell(n_cable=5)
    rc, msg = _create(m, seed=99)
    assert rc == HS_EINVAL and "seed" in msg
    rc, msg = _create(m, dt=-1.0)
    assert rc == HS_EINVAL and "dt" in msg
    bad = models.config1_cell(n_cable=5)
    bad.parent[3] = 3
    rc, msg = _create(bad)
    assert rc == HS_EINVAL
    cyc = models.config1_cell(n_cable=5)
    cyc.parent[0] = 5          # soma's parent is the last segment: a loop
    rc, msg = _create(cyc)
    assert rc == HS_EINVAL and "tree" in msg
    g = models.config1_cell(n_cable=5)
    g.chan_xgate[0] = 17
    rc, msg = _create(g)
    assert rc == HS_EINVAL and "gate" in msg
    rc, msg = _create(m, prec=HS_PREC_MIXED)
    assert rc == HS_ENOTSUP


def test_valid_model_without_gpu_reports_device_error():
    if _native.load().hs_device_count() > 0:
        pytest.skip("a GPU is present")
    rc, msg = _create(models.config1_cell(n_cable=5))
    assert rc == HS_EDEVICE


def test_empty_batch_is_refused_before_any_device_call():
    """hs_batch_create with no cells returns HS_EINVAL (checked before the
    device is touched, so this holds on a machine without a GPU)."""
    from moose_gb300 import _native
    from moose_gb300.batch import Batch
    with pytest.raises(_native.HsError):
        Batch([], 25e-6)


def test_group_and_cluster_calls_check_their_arguments():
    """hs_process_group and hs_set/get_cluster_ctas validate on the host
    (no device call), as every other entry point does."""
    L = _native.load()
    assert L.hs_process_group(None, 0, 10) == 0                 # an empty group is a no-op
    assert L.hs_process_group(None, 2, 10) == HS_EINVAL
    two = (C.c_void_p * 2)(None, None)
    assert L.hs_process_group(two, 2, 10) == HS_EINVAL          # null members
    assert L.hs_set_cluster_ctas(None, 2) == HS_EINVAL
    out = C.c_uint32()
    assert L.hs_get_cluster_ctas(None, C.byref(out)) == HS_EINVAL
    from moose_gb300.hsolve import HSolve, process_group
    h = HSolve(models.config1_cell(n_cable=5))
    with pytest.raises(ValueError):
        process_group([h], 10)                                   # no target set


def test_tick_builds_its_handle_array_once(monkeypatch):
    """moose_gb300.hsolve.Tick passes hs_process_group the members' handles
    in order, builds the array once, and again when a member's solver was
    replaced (a fake library records the calls: no GPU)."""
    from moose_gb300 import hsolve

    class S:
        def __init__(self, v):
            self._h = C.c_void_p(v)

    calls = []

    class Fake:
        def hs_process_group(self, arr, n, k):
            calls.append((id(arr), [arr[i] for i in range(n)], n, k))
            return 0

    monkeypatch.setattr(hsolve._native, "load", lambda: Fake())
    ss = [S(0x1000 + 16 * i) for i in range(5)]
    t = hsolve.Tick(ss)
    t.process()
    t.process(3)
    assert calls[0][1] == [0x1000 + 16 * i for i in range(5)] and calls[0][2:] == (5, 1)
    assert calls[1][0] == calls[0][0] and calls[1][3] == 3          # the same array
    ss[2]._h = C.c_void_p(0x9000)                                    # a new target
    t.process()
    assert calls[2][1][2] == 0x9000
    ss[4]._h = None
    with pytest.raises(ValueError):
        t.process()
