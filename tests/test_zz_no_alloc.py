"""hs_batch_set_inject_at (inject writes from fixed storage, no allocation)
against the regular path hs_batch_inject_targets + hs_batch_set_inject:
after each of two calls in a row, and steps in between, every compartment's
Vm is identical (tolerance: exact -- both write the same values to the same
solver slots).  Collected last so that it also runs after the other tests."""
import ctypes as C

import numpy as np
import pytest

from moose_gb300 import _native, models
from moose_gb300.abi import HS_EINVAL, HS_PREC_FP64, HS_PREC_MIXED, HS_ECAPACITY
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


def _device_free_bytes():
    """Free device memory from the driver (the library's primary context is
    current on this thread), or None where the driver call is unavailable."""
    try:
        cu = C.CDLL("libcuda.so.1")
    except OSError:
        return None
    free, total = C.c_size_t(), C.c_size_t()
    if cu.cuMemGetInfo_v2(C.byref(free), C.byref(total)) != 0:
        return None
    return free.value


def test_set_inject_at_allocates_nothing_and_checks_targets():
    """Repeated calls leave the device's free memory where it was (the
    entry point's purpose: it allocates nothing); targets outside the batch
    are refused with HS_EINVAL and change nothing; n == 0 is a no-op."""
    cs = cells(6, 17)
    b = Batch(cs, DT, HS_PREC_FP64)
    b.reinit(DT)
    b.process(50)
    L = _native.load()
    pu, pd = C.POINTER(C.c_uint32), C.POINTER(C.c_double)
    ids = np.arange(len(cs), dtype=np.uint32)
    soma = np.zeros(len(cs), np.uint32)
    vals = np.full(len(cs), 0.5e-9)

    def call(c, m, v, n=None):
        return L.hs_batch_set_inject_at(b._h, c.ctypes.data_as(pu), m.ctypes.data_as(pu),
                                        v.ctypes.data_as(pd), len(v) if n is None else n)

    assert call(ids, soma, vals) == 0, L.hs_last_error()     # first call: symbol lookup
    before = _device_free_bytes()
    for k in range(20):
        assert call(ids, soma, vals * (1 + 0.01 * k)) == 0, L.hs_last_error()
    after = _device_free_bytes()
    if before is not None and after is not None:
        assert after >= before, (before, after)
    vm0 = [b.vm(i).copy() for i in range(len(cs))]
    bad_cell = ids.copy()
    bad_cell[3] = len(cs)
    assert call(bad_cell, soma, vals) == HS_EINVAL
    bad_compt = soma.copy()
    bad_compt[2] = 100_000
    assert call(ids, bad_compt, vals) == HS_EINVAL
    assert call(ids, soma, vals, n=0) == 0
    # nothing was written by the refused or empty calls: stepping from here
    # matches a twin batch given only the last accepted values
    twin = Batch(cs, DT, HS_PREC_FP64)
    twin.reinit(DT)
    twin.process(50)
    twin.inject_targets(ids, soma)
    twin.set_inject(vals * (1 + 0.01 * 19))
    for i in range(len(cs)):
        assert np.array_equal(b.vm(i), vm0[i])
    for x in (b, twin):
        x.process(100)
    for i in range(len(cs)):
        assert np.array_equal(b.vm(i), twin.vm(i)), i
