"""Scheduling logic of the serving loop on a virtual clock (no GPU)."""
import numpy as np
import pytest

from raytracer_3d_gb300.serve import FakeExecutor, Request, Server, poisson_requests


class _Exp:
    def __init__(self, cells):
        self.cells = cells


def _reqs(spec):
    return [Request(i, _Exp(c), s, t, cells=c) for i, (c, s, t) in enumerate(spec)]


def test_every_request_gets_exactly_its_steps():
    reqs = _reqs([(1000, 50, 0.0), (2000, 120, 0.0), (500, 7, 0.001), (800, 300, 0.002), (100, 1, 0.5)])
    rep = Server(FakeExecutor(rate=1e6), budget_bytes=1e9, chunk_max=25).run(reqs)
    for r in reqs:
        assert r.result == r.steps
        assert r.finished is not None and r.finished >= r.arrival
    assert rep.cell_updates == sum(r.cells * r.steps for r in reqs)


def test_budget_is_respected_and_admission_is_fifo():
    # each request needs 36+72 B/cell while setting up; budget fits two at a time
    reqs = _reqs([(1000, 40, 0.0)] * 6)
    budget = 2 * 36 * 1000 + 72 * 1000 + 1
    ex = FakeExecutor(rate=1e6)
    rep = Server(ex, budget_bytes=budget, chunk_max=10).run(reqs)
    assert rep.peak_bytes <= budget
    adm = [r.admitted for r in reqs]
    assert adm == sorted(adm)
    assert max(len(ids) for _, ids, _ in ex.log) <= 2


def test_late_arrival_joins_running_batch():
    reqs = _reqs([(1000, 200, 0.0), (1000, 20, 0.001)])
    ex = FakeExecutor(rate=1e7, launch=1e-4)
    Server(ex, budget_bytes=1e9, chunk_max=10).run(reqs)
    together = [ids for _, ids, _ in ex.log if len(ids) == 2]
    assert together, "the second request never shared a chunk with the first"
    assert reqs[1].finished < reqs[0].finished


def test_request_larger_than_budget_is_rejected():
    with pytest.raises(ValueError):
        Server(FakeExecutor(), budget_bytes=1e3).run(_reqs([(1000, 5, 0.0)]))


def test_percentiles_and_poisson_generator():
    reqs = poisson_requests(40, rate=20.0, seed=3, steps_range=(5, 30), spatial=(4, 6), spectral=(4, 6))
    gaps = np.diff([0.0] + [r.arrival for r in reqs])
    assert 0.02 < gaps.mean() < 0.09
    assert all(5 <= r.steps <= 30 for r in reqs)
    for r in reqs:
        r.cells = 1000
    rep = Server(FakeExecutor(rate=1e6), budget_bytes=1e9, chunk_max=8).run(reqs)
    s = rep.summary()
    assert s["completed"] == 40
    assert s["p50_s"] <= s["p99_s"]
