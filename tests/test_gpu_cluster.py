"""Forests stepped by thread-block clusters (cluster_ctas >= 2): the CTAs of
a cluster share the assembly of each forest, rank 0 eliminates and
substitutes back.  Every node's arithmetic is the one-CTA step's, so a
clustered batch is bit-identical to the same cells in the default layout:
Vm, Ca, traces and spikes, with stop steps (the serving kernel) and
synapses."""
import numpy as np
import pytest

from moose_gb300 import _native, models
from moose_gb300.abi import HS_PREC_FP64, HS_PREC_MIXED
from moose_gb300.batch import Batch

pytestmark = pytest.mark.gpu

DT = 25e-6


def _cells():
    kca = models.kca_2d_tables(vdivs=300, cadivs=300)
    cells = []
    for i, n in enumerate((9000, 4200, 300, 1200, 60, 2500)):
        rng = np.random.default_rng([41, i])
        parent, d, L = models.branched_morphology(rng, n, 0.5, 4)
        cells.append(models.active_cell(parent, d, L, inject=float(rng.uniform(0.4e-9, 1.2e-9)), n_syn=30,
                                        rng=rng, t_end=0.05, kca_tables=kca, syn_rate=40.0))
    return cells


def _run(cells, **tuning):
    b = Batch(cells, DT, HS_PREC_MIXED, steps_per_launch=100, **tuning)
    n = len(cells)
    b.record(np.arange(n), np.zeros(n, np.uint32), 10, 200)
    b.set_stop_steps([1500, 1500, 900, 1500, 1500, 1200])
    b.reinit(DT)
    for _ in range(3):
        b.process(500)
    b.sync()
    out = dict(vm=[b.vm(i) for i in range(n)], ca=[b.ca(i) for i in range(n)], trace=b.trace()[0],
               spikes=b.spikes(), ctas=b.info()["n_ctas"], forests=b.info()["n_forests"])
    b.close()
    return out


@pytest.mark.parametrize("ctas", [2, 4, 8])
def test_clustered_batch_bit_identical_to_one_cta(ctas):
    cells = _cells()
    ref = _run(cells)
    got = _run(cells, cluster_ctas=ctas)
    assert got["ctas"] % ctas == 0
    for i in range(len(cells)):
        assert np.array_equal(got["vm"][i], ref["vm"][i]), i
        assert np.array_equal(got["ca"][i], ref["ca"][i]), i
    assert np.array_equal(got["trace"], ref["trace"])
    spikes = lambda sp: sorted(zip(sp[0].tolist(), sp[1].tolist(), sp[2].tolist()))
    assert spikes(got["spikes"]) == spikes(ref["spikes"])
    assert len(ref["spikes"][2]) > 0


def test_cluster_option_is_checked():
    cells = _cells()[:2]
    with pytest.raises(_native.HsError):
        Batch(cells, DT, HS_PREC_MIXED, cluster_ctas=9)
    with pytest.raises(_native.HsError):
        Batch(cells, DT, HS_PREC_FP64, cluster_ctas=2)
