"""Restart through the GPU library: rt_get_tendency returns the dE and meanfl
the oracle's integrate leaves behind (bit-identical in binary64), and a run
continued from a restart file (restart.f90) equals the uninterrupted run."""
import dataclasses

import numpy as np
import pytest

from harness import ONX, build_oracle, configs, interior, max_rel
from raytracer_3d_gb300 import restart

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()


def _flux(m):
    P = tuple(m.n[a] + 2 * ONX for a in (0, 1, 3, 4, 5))
    return "flux", np.asfortranarray(np.random.default_rng(9).uniform(0.0, 1e-3, size=P))


CASES = {
    "shear_mini": lambda: configs.shear_mini(),
    "column_1d": lambda: configs.column_1d(fac=1),
    "stretched": lambda: configs.stretched_mini(),
    "forced": lambda: dataclasses.replace(configs.shear_mini(n=(6, 4, 6, 4, 4, 4)), forcing=_flux),
}


@pytest.mark.parametrize("name", list(CASES))
def test_tendency_bit_identical(name):
    exp = CASES[name]()
    m = configs.build_model(exp, "fp64")
    o = build_oracle(exp)
    sl = interior(exp.n)
    try:
        dE0, mf0 = m.get_tendency()             # before a step: zeros
        assert not dE0.any() and not mf0.any()
        m.integrate(3)
        o.integrate(3)
        dE, mf = m.get_tendency()
        assert np.array_equal(dE[sl], o.dE[sl]), max_rel(dE[sl], o.dE[sl])
        assert np.array_equal(mf[sl], o.meanfl[sl])
    finally:
        m.close()


def test_tendency_fp32_within_tolerance():
    exp = configs.shear_mini()
    m = configs.build_model(exp, "fp32")
    o = build_oracle(exp)
    sl = interior(exp.n)
    try:
        m.integrate(2)
        o.integrate(2)
        dE, mf = m.get_tendency()
        assert max_rel(dE[sl], o.dE[sl]) <= 1e-4
        assert max_rel(mf[sl], o.meanfl[sl]) <= 1e-5
    finally:
        m.close()


@pytest.mark.parametrize("name", ["shear_mini", "forced"])
def test_continued_run_equals_uninterrupted(name, tmp_path):
    exp = CASES[name]()
    a = configs.build_model(exp, "fp64")
    b = configs.build_model(exp, "fp64")
    o = build_oracle(exp)
    sl = interior(exp.n)
    try:
        a.integrate(4)
        o.integrate(4)
        path = restart.write_restart(a, str(tmp_path))
        dims, itt, E, dE, mf = restart.read_arrays(path, n=exp.n)
        assert itt == 4 and (tmp_path / "ritt").read_text().split() == ["4"]
        assert np.array_equal(E[sl], o.E[sl]) and np.array_equal(dE[sl], o.dE[sl])
        assert np.array_equal(mf[sl], o.meanfl[sl])
        b.E[...] = 0.0
        got = restart.read_restart(b, str(tmp_path))
        assert got is not None and got[0] == 4 and b.itt == 4
        a.integrate(3)
        b.integrate(3)
        assert np.array_equal(a.get_state()[sl].copy(), b.get_state()[sl])
    finally:
        a.close()
        b.close()
