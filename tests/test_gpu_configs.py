"""The workloads at their full sizes and lengths.

* 32^6 plain binary64 (the bench workload): one step of each bit-exact
  schedule from the same state gives the same field bit for bit, and the
  fast schedule is within 1e-12 relative L-infinity of them.
* 32^6 binary32, 1000 steps, against binary64 (the fast schedule, itself
  held to 1e-12 per step of the reference's arithmetic): relative L2
  <= 1e-5 and relative total-energy drift <= 1e-9.
* the 48-member binary32 ensemble, 500 steps in one batch, against every
  member run alone in binary64: L2 <= 1e-5 per member; the energy drift of
  the ensemble and of every member within 1e-9 or four standard deviations
  of the binary32 update's unbiased rounding noise, whichever is larger (a
  member of 8^3 x 8^3 cells whose packet covers a few thousand cells has a
  noise of a few 1e-9 over 500 steps).

These runs hold up to about 210 GB of device memory and take minutes; each
binary64 handle is closed before the binary32 one is built."""
import numpy as np
import pytest

from harness import (build_point_oracle, configs, energy_sum, error_norms, max_rel, rounding_noise_bound,
                     sample_cells, vol_weights)

pytestmark = pytest.mark.gpu

FP64_STEP_TOL = 1e-12
FP32_L2_TOL = 1e-5        # relative L2 of E against binary64
FP32_DRIFT_TOL = 1e-9     # relative total-energy difference against binary64


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()


def test_jet_large_schedules_agree_at_32e6():
    exp = configs.jet_large()
    m = configs.build_model(exp, "fp64", padded=False)
    try:
        E0 = m.E.copy(order="F")
        out = {}
        for sched in ("tma", "split", "fast"):
            m.E = E0
            m.set_state()
            m.set_tuning(sched, 8, 256)
            m.integrate(1)
            out[sched] = m.get_state()
        assert np.array_equal(out["tma"], out["split"])
        rel = max_rel(out["fast"], out["split"])
        print("32^6 binary64: tma == split bit for bit; fast within %.2e" % rel)
        assert rel <= FP64_STEP_TOL
    finally:
        m.close()


def test_jet_large_cells_against_the_oracle_at_32e6():
    """1500 cells of one bit-exact step at 32^6 (half of them on a boundary
    plane: open faces, z walls under reflection, the edges of the spectral
    axes) against the oracle's per-cell restatement of the reference's
    update, from the same pre-step state: bit-identical; the fast schedule
    within 1e-12 of it"""
    exp = configs.jet_large()
    m = configs.build_model(exp, "fp64", padded=False)
    po = None
    try:
        m.set_tuning("split", 8, 256)
        m.integrate(10)          # outflow and refraction have built gradients by now
        E0 = m.get_state()
        m.integrate(1)
        E1 = m.get_state()
        po = build_point_oracle(exp, m.dt)
        cells = sample_cells(exp.n, 1500, np.random.default_rng(99))
        ref = po.point_steps(E0, cells)
        idx = tuple((cells - 1).T)
        got = E1[idx]
        assert np.array_equal(got, ref), float(np.max(np.abs(got - ref)))
        m.E = E0
        m.set_state()
        m.set_tuning("fast", 8, 256)
        m.integrate(1)
        fast = m.get_state()[idx]
        rel = float(np.max(np.abs(fast - ref))) / float(np.max(np.abs(E1)))
        print("32^6: %d cells of the split step equal the per-cell oracle; fast within %.2e" % (len(cells), rel))
        assert rel <= FP64_STEP_TOL
    finally:
        if po is not None:
            po.close()
        m.close()


def test_jet_large_fp32_1000_steps_at_32e6():
    exp = configs.jet_large()
    steps = 1000
    m64 = configs.build_model(exp, "fp64", padded=False)
    try:
        w = vol_weights(m64)
        m64.E = np.asfortranarray(m64.E.astype(np.float32).astype(np.float64))   # the binary32 form's input
        m64.set_state()
        e_start = energy_sum(m64.E, w)
        m64.set_tuning("fast", 8, 256)
        m64.integrate(steps)
        ref = m64.get_state()
    finally:
        m64.close()
    m32 = configs.build_model(exp, "fp32", padded=False)
    try:
        m32.set_tuning("w2z", 8, 512, 1)
        m32.integrate(steps)
        got = m32.get_state()
    finally:
        m32.close()
    assert np.isfinite(got).all()
    l2, linf = error_norms(got, ref)
    e64, e32 = energy_sum(ref, w), energy_sum(got, w)
    drift = abs(e32 - e64) / abs(e64)
    print("jet_large 32^6, %d steps, binary32 against binary64: L2 %.3e  Linf %.3e  energy %.3e  "
          "(binary64 energy change over the run %.3e)" % (steps, l2, linf, drift, abs(e64 - e_start) / abs(e_start)))
    assert l2 <= FP32_L2_TOL
    assert drift <= FP32_DRIFT_TOL


def test_ensemble48_fp32_500_steps_against_fp64():
    from raytracer_3d_gb300.batch import Batch
    rng = np.random.default_rng(2024)
    exps = [configs.ensemble_member(rng, steps=500) for _ in range(48)]
    steps = 500
    models = [configs.build_model(e, "fp32", padded=False) for e in exps]
    b = Batch(models)
    try:
        b.set_tuning(8, 512, 1, 16)
        b.set_persistent(512)
        b.integrate(steps)
        b.sync()
        got = [m.get_state() for m in models]
        weights = [vol_weights(m) for m in models]
    finally:
        b.close()
        for m in models:
            m.close()
    worst = {"l2": 0.0, "linf": 0.0, "drift": 0.0, "excess": 0.0}
    tot32 = tot64 = var = 0.0
    for e, g, w in zip(exps, got, weights):
        m = configs.build_model(e, "fp64", padded=False)
        try:
            m.E = np.asfortranarray(m.E.astype(np.float32).astype(np.float64))   # the member's binary32 input
            m.set_state()
            m.set_tuning("fast", 8, 256)
            m.integrate(steps)
            ref = m.get_state()
        finally:
            m.close()
        l2, linf = error_norms(g, ref)
        e64, e32 = energy_sum(ref, w), energy_sum(g, w)
        tot32 += e32
        tot64 += e64
        noise = rounding_noise_bound(ref, w, steps)        # 4 standard deviations, relative
        var += (noise / 4 * e64) ** 2
        drift = abs(e32 - e64) / abs(e64)
        worst["l2"] = max(worst["l2"], l2)
        worst["linf"] = max(worst["linf"], linf)
        worst["drift"] = max(worst["drift"], drift)
        # a small member's own unbiased rounding noise may exceed 1e-9
        worst["excess"] = max(worst["excess"], drift / max(FP32_DRIFT_TOL, noise))
    ens = abs(tot32 - tot64) / abs(tot64)
    # the ensemble's own rounding noise: the members' independent deviations
    # add in quadrature, weighted by their energies (the small members carry
    # most of it: a packet of a few cells per axis on a coarse grid)
    ens_noise = 4 * var ** 0.5 / abs(tot64)
    print("48-member ensemble, %d steps, binary32 batch against binary64 alone: ensemble energy %.3e "
          "(noise allowance %.2e); worst member L2 %.3e  Linf %.3e  energy %.3e (%.2f of its allowance)"
          % (steps, ens, ens_noise, worst["l2"], worst["linf"], worst["drift"], worst["excess"]))
    assert worst["l2"] <= FP32_L2_TOL
    assert ens <= max(FP32_DRIFT_TOL, ens_noise)
    assert worst["excess"] <= 1.0
