"""Bottom forcing on the GPU (rt_set_forcing; set_forcing of lee1.f90:193-229
and critical_gm1.f90:119-141) against the oracle: the binary64 form is
bit-identical after every step, the binary32 form stays within the stated
tolerance, and a batch applies each member's own forcing."""
import dataclasses

import numpy as np
import pytest

from harness import ONX, build_oracle, configs, interior, max_rel

pytestmark = pytest.mark.gpu

FP32_REL = 1e-5     # relative L-inf after a few steps, binary32 form against the binary64 oracle


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()


def _random_forcing(kind, seed, scale=1e-3):
    def forcing(m):
        P = tuple(m.n[a] + 2 * ONX for a in (0, 1, 3, 4, 5))
        rng = np.random.default_rng(seed)
        return kind, np.asfortranarray(rng.uniform(0.0, scale, size=P))
    return forcing


CASES = {
    "lee_wave_flux": lambda: configs.lee_wave_flux(fac=1),
    "critical_gm_relax": lambda: configs.critical_gm_relax(fac=0.5),
    "shear_flux": lambda: dataclasses.replace(configs.shear_mini(), forcing=_random_forcing("flux", 5)),
    "shear_relax": lambda: dataclasses.replace(configs.shear_mini(n=(8, 8, 8, 4, 4, 6)),
                                               forcing=_random_forcing("relax", 6)),
    "ragged_relax": lambda: dataclasses.replace(configs.shear_mini(n=(7, 3, 5, 2, 6, 4), upper=False),
                                                forcing=_random_forcing("relax", 7)),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("variant", ["tma", "plane", "cell", "split"])
def test_forced_steps_bit_identical(name, variant):
    exp = CASES[name]()
    m = configs.build_model(exp, "fp64")
    m.set_tuning(variant)
    o = build_oracle(exp)
    sl = interior(exp.n)
    try:
        assert m.dt == o.dt
        for s in range(4):
            m.integrate(1)
            o.integrate(1)
            got = m.get_state()[sl]
            assert np.array_equal(got, o.E[sl]), (s, max_rel(got, o.E[sl]))
        assert o.E[sl].any()
    finally:
        m.close()


@pytest.mark.parametrize("name", ["shear_flux", "shear_relax", "critical_gm_relax"])
def test_forced_budget_matches_diagnose(name):
    exp = CASES[name]()
    m = configs.build_model(exp, "fp64")
    o = build_oracle(exp)
    try:
        m.integrate(3)
        o.integrate(3)
        b, f = m.diagnose()
        bo = o.diagnose()
        sl3 = interior(exp.n[:3])
        assert np.array_equal(f["E_int"][sl3], o.E_int[sl3])
        # the sums are reduced in another order than the oracle's: the
        # difference is bounded by n*eps*sum|terms| (the forced column
        # cancels to 1e-10 of its terms)
        sl = interior(exp.n)
        vol = np.ones((1,) * 6)
        for a, ax in enumerate("xyzklm"):
            shp = [1] * 6
            shp[a] = exp.n[a]
            vol = vol * o.grid[ax]["dt"][ONX:ONX + exp.n[a]].reshape(shp)
        bound = exp.cells * np.finfo(np.float64).eps
        terms = {"eint": np.abs(o.dE[sl] * vol).sum(), "mflint": np.abs(o.meanfl[sl] * vol).sum()}
        for k, t in terms.items():
            assert abs(b[k] - bo[k]) <= bound * t, (k, b[k], bo[k], t)
        # boundary sums cancel too (faces of both flow directions)
        scale = sum(terms.values()) + sum(abs(bo[k]) for k in bo if k.startswith("bfl"))
        for k in ("bfl_zs", "bfl_ze"):
            assert abs(b[k] - bo[k]) <= 1e-12 * abs(bo[k]) + 1e-15 * scale, (k, b[k], bo[k])
    finally:
        m.close()


@pytest.mark.parametrize("variant", ["tma", "w2z", "w3", "w6", "group"])
def test_forced_fp32_within_tolerance(variant):
    """8x8 planes with 256 threads: every listed kernel takes the case"""
    exp = CASES["shear_relax"]()
    o = build_oracle(exp)
    m = configs.build_model(exp, "fp32")
    m.set_tuning(variant, 8, 256)
    sl = interior(exp.n)
    try:
        m.integrate(5)
        o.integrate(5)
        rel = max_rel(m.get_state()[sl], o.E[sl])
        assert rel <= FP32_REL, rel
    finally:
        m.close()


def test_forcing_off_equals_unforced():
    exp = CASES["shear_flux"]()
    m = configs.build_model(exp, "fp64")
    m.set_forcing("none")
    o = build_oracle(configs.shear_mini())
    sl = interior(exp.n)
    try:
        m.integrate(3)
        o.integrate(3)
        assert np.array_equal(m.get_state()[sl], o.E[sl])
    finally:
        m.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_applies_each_members_forcing(precision):
    """Forced and unforced members in one batch give each member exactly
    its result alone, also when a forcing changes between batch calls."""
    from raytracer_3d_gb300.batch import Batch
    rng = np.random.default_rng(21)
    exps = [configs.ensemble_member(rng, steps=6, spatial=(4, 8), spectral=(4, 6)) for _ in range(4)]
    exps[0] = dataclasses.replace(exps[0], forcing=_random_forcing("flux", 1))
    exps[2] = dataclasses.replace(exps[2], forcing=_random_forcing("relax", 2))

    def alone(e, switch_off):
        m = configs.build_model(e, precision)
        m.integrate(3)
        if switch_off:
            m.set_forcing("none")
        m.integrate(3)
        out = m.get_state().copy()
        m.close()
        return out

    refs = [alone(e, j == 0) for j, e in enumerate(exps)]
    models = [configs.build_model(e, precision) for e in exps]
    b = Batch(models)
    b.set_tuning(8, 256, 0, 2)
    b.integrate(3)
    models[0].set_forcing("none")
    b.integrate(3)
    for e, m, ref in zip(exps, models, refs):
        sl = interior(e.n)
        assert np.array_equal(m.get_state()[sl], ref[sl]), e.n
    b.close()
    for m in models:
        m.close()
