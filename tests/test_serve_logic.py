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


# ---- failure isolation: injected on the host, no GPU involved ----
def test_failed_setup_leaves_the_others_exact():
    reqs = _reqs([(1000, 40, 0.0), (2000, 30, 0.0), (500, 25, 0.001), (800, 60, 0.002)])
    ex = FakeExecutor(rate=1e6, fail_admit={1})
    rep = Server(ex, budget_bytes=1e9, chunk_max=10).run(reqs)
    assert reqs[1].status == "failed" and "injected set-up failure" in reqs[1].error
    for r in (reqs[0], reqs[2], reqs[3]):
        assert r.status == "done" and r.result == r.steps
    assert all(1 not in ids for _, ids, _ in ex.log)
    s = rep.summary()
    assert (s["completed"], s["failed"], s["cancelled"]) == (3, 1, 0)
    assert rep.cell_updates == sum(r.cells * r.steps for r in reqs if r.status == "done")


def test_failed_setup_returns_its_memory():
    # the budget holds one request; the first fails, the second must still run
    reqs = _reqs([(1000, 10, 0.0), (1000, 10, 0.0)])
    budget = 36 * 1000 + 72 * 1000 + 1
    rep = Server(FakeExecutor(rate=1e6, fail_admit={0}), budget_bytes=budget, chunk_max=5).run(reqs)
    assert reqs[0].status == "failed" and reqs[1].status == "done" and reqs[1].result == 10
    assert rep.peak_bytes <= budget


def test_failed_result_read_is_contained():
    reqs = _reqs([(1000, 20, 0.0), (1000, 20, 0.0), (1000, 50, 0.0)])
    ex = FakeExecutor(rate=1e6, fail_retire={0})
    Server(ex, budget_bytes=1e9, chunk_max=10).run(reqs)
    assert reqs[0].status == "failed" and reqs[0].result is None
    assert reqs[1].result == 20 and reqs[2].result == 50


@pytest.mark.parametrize("when", ["queued", "running"])
def test_cancelled_request_leaves_without_perturbing_the_others(when):
    # 1000 cells at 1e6 cells/s: 1 ms per step per member
    reqs = _reqs([(1000, 100, 0.0), (1000, 100, 0.0), (1000, 30, 0.0), (1000, 80, 0.05)])
    if when == "queued":
        reqs[3].cancel_at = 0.01          # before it arrives
    else:
        reqs[1].cancel_at = 0.03          # mid-flight
    ex = FakeExecutor(rate=1e6)
    rep = Server(ex, budget_bytes=1e9, chunk_max=10).run(reqs)
    gone = reqs[3] if when == "queued" else reqs[1]
    assert gone.status == "cancelled" and gone.result is None and gone.finished is None
    for r in reqs:
        if r is not gone:
            assert r.status == "done" and r.result == r.steps
    if when == "running":
        assert ex.discarded == [1]
        last = max(t for t, ids, _ in ex.log if 1 in ids)
        assert last <= 0.03 + 0.05        # left at a chunk boundary after cancel_at
    assert rep.summary()["cancelled"] == 1


def test_cancellation_frees_budget_for_the_queue():
    # budget for one request at a time; cancelling the first lets the second start early
    reqs = _reqs([(1000, 1000, 0.0), (1000, 10, 0.0)])
    reqs[0].cancel_at = 0.02
    budget = 36 * 1000 + 72 * 1000 + 1
    Server(FakeExecutor(rate=1e6), budget_bytes=budget, chunk_max=10).run(reqs)
    assert reqs[0].status == "cancelled"
    assert reqs[1].status == "done" and reqs[1].admitted < 0.1
