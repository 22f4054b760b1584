"""Failure detection on the GPU without a GPU fault.

* A device-side wait that can never complete gives up after its poll limit,
  raises the status flag and returns; the context stays usable
  (rt_selftest_wait_timeout runs the step kernels' wait code with a short
  limit on mbarriers that nothing completes: no trap, no fault, no copy in
  flight).
* In the serving loop a request whose set-up fails and a request the client
  cancels mid-flight leave without changing any other request's result.
"""
import ctypes
import dataclasses
import time

import numpy as np
import pytest

from harness import build_oracle, configs, interior

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()


def test_bounded_wait_gives_up_and_the_context_survives():
    from raytracer_3d_gb300 import _lib
    lib = _lib.load()
    status, completed = ctypes.c_int(-1), ctypes.c_int(-1)
    t0 = time.perf_counter()
    assert lib.rt_selftest_wait_timeout(ctypes.byref(status), ctypes.byref(completed)) == 0
    elapsed = time.perf_counter() - t0
    assert status.value == 1 and completed.value == 0
    assert elapsed < 30.0
    # the same context still steps correctly, with a clean status
    exp = configs.shear_mini()
    m = configs.build_model(exp, "fp64")
    o = build_oracle(exp)
    try:
        m.integrate(2)
        o.integrate(2)
        sl = interior(exp.n)
        assert np.array_equal(m.get_state()[sl], o.E[sl])
    finally:
        m.close()


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_serving_isolates_a_failed_and_a_cancelled_request(precision):
    from raytracer_3d_gb300.serve import GpuExecutor, Request, Server
    rng = np.random.default_rng(5)
    exps = [configs.ensemble_member(rng, steps=int(rng.integers(5, 30)), spatial=(4, 8), spectral=(4, 6))
            for _ in range(5)]
    # request 1 cannot be created (nk odd, parallel_mpi.f90:16-25); request 3
    # would run for a long time and is cancelled after a second
    bad = dataclasses.replace(exps[1], n=(4, 4, 4, 3, 4, 4))
    long_run = dataclasses.replace(exps[3], steps=10 ** 6)
    exps[1], exps[3] = bad, long_run
    reqs = [Request(i, e, e.steps, 0.001 * i, cells=e.cells) for i, e in enumerate(exps)]
    reqs[3].cancel_at = 1.0
    ex = GpuExecutor(precision=precision, batch_tuning=(8, 256, 0, 2))
    try:
        rep = Server(ex, budget_bytes=20e9, chunk_max=4, setup_workers=2).run(reqs)
    finally:
        ex.close()
    assert reqs[1].status == "failed" and "rt_create" in reqs[1].error
    assert reqs[3].status == "cancelled" and reqs[3].result is None
    s = rep.summary()
    assert (s["completed"], s["failed"], s["cancelled"]) == (3, 1, 1)
    for i in (0, 2, 4):
        e = exps[i]
        m = configs.build_model(e, precision, padded=False)
        m.integrate(e.steps)
        ref = m.get_state()
        m.close()
        assert reqs[i].status == "done"
        assert np.array_equal(reqs[i].result, ref), i
