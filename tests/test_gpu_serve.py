"""Serving loop on the GPU: continuous batching of requests that arrive
while others run; each result must equal the same integration run alone."""
import numpy as np
import pytest

from harness import configs, interior

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()


def test_served_results_equal_alone():
    from raytracer_3d_gb300.serve import GpuExecutor, Server, poisson_requests
    reqs = poisson_requests(10, rate=200.0, seed=21, steps_range=(3, 40), spatial=(4, 6, 8), spectral=(4, 6))
    ex = GpuExecutor("fp32")
    rep = Server(ex, budget_bytes=2e9, chunk_max=8).run(reqs)
    ex.close()
    s = rep.summary()
    assert s["completed"] == len(reqs)
    assert rep.chunks > 1
    for r in reqs:
        m = configs.build_model(r.exp, "fp32")
        m.integrate(r.steps)
        alone = m.get_state()
        sl = interior(r.exp.n)
        assert r.result.shape == tuple(r.exp.n)       # interior, binary32
        assert np.array_equal(r.result.astype(np.float64), alone[sl]), r.rid
        m.close()


def test_small_budget_serialises_but_completes():
    from raytracer_3d_gb300.serve import GpuExecutor, Server, bytes_per_cell, poisson_requests
    reqs = poisson_requests(4, rate=1000.0, seed=2, steps_range=(2, 6), spatial=(4,), spectral=(4,))
    res, tmp = bytes_per_cell("fp32")
    budget = (res + tmp) * max(r.cells for r in reqs) * 1.01
    ex = GpuExecutor("fp32")
    rep = Server(ex, budget_bytes=budget, chunk_max=4).run(reqs)
    ex.close()
    assert rep.summary()["completed"] == 4
    assert rep.peak_bytes <= budget


def test_autotuner_picks_a_schedule_without_changing_results(tmp_path, monkeypatch):
    monkeypatch.setenv("RT_TUNE_CACHE", str(tmp_path / "tune.json"))
    from raytracer_3d_gb300.autotune import tune_model
    exp = configs.shear_mini(n=(8, 8, 8, 6, 6, 8))
    ref = configs.build_model(exp, "fp32")
    ref.integrate(4)
    E_ref = ref.get_state().copy()
    ref.close()
    m = configs.build_model(exp, "fp32")
    best, table = tune_model(m, reps=1)
    assert len(table) >= 4 and best == table[0][0]
    m.integrate(4)
    sl = interior(exp.n)
    assert np.array_equal(m.get_state()[sl], E_ref[sl])
    # cached second call
    best2, _ = tune_model(m)
    assert best2 == best
    m.close()
