"""Serving loop host logic on the CPU: admission against the memory budget,
continuous batching of arrivals into cohorts, per-request completion and
latency accounting.  The device cohort is replaced by a stand-in that
advances its cells by the chunk without a GPU."""
import numpy as np

from moose_gb300 import serve


class _Cell:
    def __init__(self, n):
        self.n_compt = n
        self.syn_compt = np.zeros(0)
        self.ev_time = np.zeros(0)
        self.gates = [(-0.1, 0.05, np.zeros(3001), np.zeros(3001))]
        self.gates2d = []


class FakeCohort:
    created = []

    def __init__(self, reqs, dt, stride, chunk, now, tuning):
        self.reqs = reqs
        self.tuning = dict(tuning)
        self.admitted = now
        self.bytes = serve.cohort_overhead(reqs[0].cell) + sum(
            serve.estimate_bytes(r.cell, r.n_steps, stride) for r in reqs)
        self.done = np.zeros(len(reqs), bool)
        self.steps = 0
        self.stride = stride
        self.vm = [[] for _ in reqs]
        self.spikes = [[] for _ in reqs]
        self.closed = False
        FakeCohort.created.append(self)

    def launch(self, chunk):
        self.steps += chunk

    def ready(self):
        return True

    def collect(self):
        fresh = [i for i, r in enumerate(self.reqs) if not self.done[i] and self.steps >= r.n_steps]
        for i in fresh:
            self.done[i] = True
            self.vm[i].append(np.arange(self.reqs[i].n_steps // self.stride + 1, dtype=float))
        return fresh

    def close(self):
        self.closed = True


def make_server(**kw):
    """A server whose clock is its tick count (arrival times are in ticks)."""
    box = []
    srv = serve.Server(25e-6, clock=lambda: float(box[0].ticks) if box else 0.0, cohort_factory=FakeCohort, **kw)
    box.append(srv)
    return srv


def test_every_request_completes_with_its_steps():
    FakeCohort.created = []
    reqs = [serve.Request(i, _Cell(100 + 10 * i), 100 * (i % 5 + 1), arrival=float(i)) for i in range(12)]
    srv = make_server(chunk=100, record_stride=10)
    res = srv.run(reqs)
    assert sorted(r.rid for r in res) == list(range(12))
    for r in res:
        assert r.finished >= r.arrival
        assert len(r.vm) == r.n_steps // 10 + 1
    # arrivals spread over ticks form several cohorts, all released at the end
    assert len(FakeCohort.created) > 1
    assert all(c.closed for c in FakeCohort.created)
    assert not srv.cohorts and not srv.waiting


def test_admission_respects_the_budget():
    FakeCohort.created = []
    cell = _Cell(1000)
    one = serve.estimate_bytes(cell, 400, 40)
    budget = serve.cohort_overhead(cell) + int(2.5 * one)
    reqs = [serve.Request(i, _Cell(1000), 400, arrival=0.0) for i in range(6)]
    srv = make_server(chunk=100, record_stride=40, budget_bytes=budget)
    res = srv.run(reqs, real_time=False)
    assert len(res) == 6
    assert srv.peak_bytes <= budget
    assert max(len(c.reqs) for c in FakeCohort.created) <= 2
    # a later request is admitted only after memory was released
    first = min(c.admitted for c in FakeCohort.created)
    assert any(c.admitted > first for c in FakeCohort.created)


def test_summary_percentiles():
    rs = [serve.Result(i, 100, 1000, 0.0, 0.0, float(i + 1), np.zeros(1), np.zeros(0)) for i in range(100)]
    s = serve.summarize(rs, 10.0, offered_rate=2000.0)
    assert s["requests"] == 100
    assert abs(s["p50_latency_s"] - 50.5) < 1e-9
    assert s["p99_latency_s"] > 99.0
    assert s["compartment_steps_per_s"] == 100 * 100 * 1000 / 10.0


def test_a_round_makes_one_cohort_per_duration_class():
    FakeCohort.created = []
    steps = [4000, 20000, 60000, 5000, 30000, 70000, 12000]
    reqs = [serve.Request(i, _Cell(200), n, arrival=0.0) for i, n in enumerate(steps)]
    srv = make_server(chunk=4000, record_stride=40, duration_classes=(16000, 40000))
    res = srv.run(reqs, real_time=False)
    assert sorted(r.rid for r in res) == list(range(len(steps)))
    classes = [{srv._class(r) for r in c.reqs} for c in FakeCohort.created]
    assert all(len(c) == 1 for c in classes)
    assert len(FakeCohort.created) == 3
    # all three were admitted in the first round
    assert len({c.admitted for c in FakeCohort.created}) == 1


def test_a_round_separates_small_and_large_cells():
    """Requests of one duration but of cells on both sides of a size
    boundary go to different cohorts, so a small cell is not held to the
    step time of a large one."""
    FakeCohort.created = []
    sizes = [150, 6000, 300, 8000, 2500]
    reqs = [serve.Request(i, _Cell(n), 4000, arrival=0.0) for i, n in enumerate(sizes)]
    srv = make_server(chunk=4000, record_stride=40, duration_classes=(16000,), size_classes=(1000, 4000))
    res = srv.run(reqs, real_time=False)
    assert sorted(r.rid for r in res) == list(range(len(sizes)))
    groups = sorted(sorted(r.cell.n_compt for r in c.reqs) for c in FakeCohort.created)
    assert groups == [[150, 300], [2500], [6000, 8000]]


def test_largest_cells_get_clusters_while_sms_are_free():
    FakeCohort.created = []
    sizes = [6000, 7000, 200]
    reqs = [serve.Request(i, _Cell(n), 4000, arrival=0.0) for i, n in enumerate(sizes)]
    srv = make_server(chunk=4000, record_stride=40, duration_classes=(16000,), size_classes=(1000, 4000),
                      cluster_ctas=4)
    srv.run(reqs, real_time=False)
    tun = {tuple(sorted(r.cell.n_compt for r in c.reqs)): c.tuning for c in FakeCohort.created}
    assert tun[(6000, 7000)].get("cluster_ctas") == 4 and tun[(6000, 7000)]["max_ctas"] == 8
    assert "cluster_ctas" not in tun[(200,)]
