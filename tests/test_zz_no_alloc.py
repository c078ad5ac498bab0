"""hs_batch_set_inject_at (inject writes from fixed storage, no allocation)
against the regular path hs_batch_inject_targets + hs_batch_set_inject:
after each of two calls in a row, and steps in between, every compartment's
Vm is identical (tolerance: exact -- both write the same values to the same
solver slots).  Collected last so that it also runs after the other tests."""
import ctypes as C

import numpy as np
import pytest

from moose_gb300 import _native, models
from moose_gb300.abi import HS_PREC_FP64, HS_PREC_MIXED, HS_ECAPACITY
from moose_gb300.batch import Batch

pytestmark = pytest.mark.gpu

DT = 25e-6


def cells(n, seed):
    kA, kB = models.kca_2d_tables(vdivs=300, cadivs=300)
    out = []
    for i in range(n):
        rng = np.random.default_rng([seed, i])
        parent, d, L = models.branched_morphology(rng, int(rng.integers(20, 200)), 0.5, 4)
        out.append(models.active_cell(parent, d, L, inject=float(rng.uniform(0.2e-9, 0.8e-9)), rng=rng,
                                      t_end=0.05, kca_tables=(kA, kB)))
    return out


@pytest.mark.parametrize("precision", [HS_PREC_MIXED, HS_PREC_FP64])
def test_set_inject_at_matches_the_registered_path(precision):
    cs = cells(10, 41)
    ids = np.arange(len(cs), dtype=np.uint32)
    soma = np.zeros(len(cs), np.uint32)
    ref = Batch(cs, DT, precision)
    new = Batch(cs, DT, precision)
    ref.inject_targets(ids, soma)
    for b in (ref, new):
        b.reinit(DT)
        b.process(100)
    L = _native.load()
    pu, pd = C.POINTER(C.c_uint32), C.POINTER(C.c_double)
    for call in range(2):
        vals = np.linspace(0.1e-9, 1.2e-9, len(cs)) * (1.0 + 0.5 * call)
        ref.set_inject(vals)
        rc = L.hs_batch_set_inject_at(new._h, ids.ctypes.data_as(pu), soma.ctypes.data_as(pu),
                                      vals.ctypes.data_as(pd), len(vals))
        assert rc == 0, L.hs_last_error()
        for b in (ref, new):
            b.process(150)
        for i in range(len(cs)):
            assert np.array_equal(new.vm(i), ref.vm(i)), (call, i)


def test_set_inject_at_rejects_too_many_writes():
    b = Batch(cells(2, 5), DT, HS_PREC_MIXED)
    b.reinit(DT)
    n = 32769
    z = np.zeros(n, np.uint32)
    v = np.zeros(n)
    L = _native.load()
    rc = L.hs_batch_set_inject_at(b._h, z.ctypes.data_as(C.POINTER(C.c_uint32)),
                                  z.ctypes.data_as(C.POINTER(C.c_uint32)),
                                  v.ctypes.data_as(C.POINTER(C.c_double)), n)
    assert rc == HS_ECAPACITY
    assert b"32768" in L.hs_last_error()
