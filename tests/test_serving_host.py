"""Scheduling of the serving loop on the host: admission against slots and the memory budget,
per-molecule retirement, size classes kept apart, results independent of the cohort."""

import time

import numpy as np

from pyseqm_gb300 import serving, workloads


class FakeCohort:
    """Stands in for a device cohort: molecule rid converges after 3 + rid % 4 iterations."""

    made = []

    def __init__(self, reqs, method, eps, form, device, large, stream, graphs=False):
        self.reqs, self.large = reqs, large
        self.bytes = sum(serving.footprint(r, form) for r in reqs)
        self.stream, self.future, self.finished = stream, None, False
        self.it = 0
        self.retired = np.zeros(len(reqs), dtype=bool)
        FakeCohort.made.append(self)

    def admit(self):
        return []

    def iterate(self, t0):
        time.sleep(0.002)
        self.it += 1
        out = []
        for m, r in enumerate(self.reqs):
            if not self.retired[m] and self.it >= 3 + r.rid % 4:
                out.append(serving.Result(r.rid, float(r.rid), 0.0, 0.0, self.it, True, None, r.arrival,
                                          time.perf_counter() - t0))
                self.retired[m] = True
        self.finished = bool(self.retired.all())
        return out

    def launches(self):
        return 0


def _requests(n, seed=0):
    mols = workloads.request_molecules(n, seed=seed, atoms=(3, 120))
    return serving.make_requests(mols, np.arange(n) * 0.001)


def test_every_request_served_once_with_its_own_iterations():
    FakeCohort.made = []
    reqs = _requests(40)
    loop = serving.ServingLoop(device="cpu", cohort_factory=FakeCohort)
    res = loop.run(reqs)
    assert [r.rid for r in res] == list(range(40))
    for r in res:
        assert r.Etot == float(r.rid) and r.iterations == 3 + r.rid % 4
        assert r.done >= r.arrival
    assert loop.cohorts == len(FakeCohort.made) > 1
    assert loop.max_concurrent >= 2  # later arrivals were admitted while earlier cohorts ran
    for c in FakeCohort.made:  # Jacobi-sized and SP2-sized molecules never share a cohort
        assert all((serving.norb_of(r.species) > 160) == c.large for r in c.reqs)


def test_budget_and_slots_bound_admission():
    FakeCohort.made = []
    reqs = _requests(30, seed=3)
    big = max(serving.footprint(r) for r in reqs)
    loop = serving.ServingLoop(device="cpu", cohort_factory=FakeCohort, budget_bytes=3 * big, max_live=(2, 1))
    res = loop.run(reqs)
    assert len(res) == 30
    assert loop.max_bytes <= 3 * big
    assert loop.max_concurrent <= 3


def test_request_stream_shape():
    mols = workloads.request_molecules(400, seed=1)
    na = np.array([s.size for s, _, _ in mols])
    assert na.min() >= 3 and na.max() <= 602
    assert 0.04 < np.mean([f for *_, f in mols]) < 0.2
    for s, c, _ in mols:
        assert np.all(s[:-1] >= s[1:]) and c.shape == (s.size, 3)
    t = workloads.poisson_arrivals(5000, 1000.0)
    assert np.all(np.diff(t) > 0) and abs(5000 / t[-1] - 1000.0) < 60.0


def test_summary_percentiles():
    res = [serving.Result(i, 0.0, 0.0, 0.0, 1, True, None, 0.0, (i + 1) * 1e-3) for i in range(100)]
    s = serving.summarize(res)
    assert abs(s["p50_ms"] - 50.5) < 1e-9 and abs(s["solves_per_s"] - 1000.0) < 1e-6
