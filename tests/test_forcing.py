"""CPU checks of the bottom forcing (set_forcing of the forced reference
configurations, lee1.f90:193-229 and critical_gm1.f90:119-141) in the
oracle, the forced experiments, and argument checks of rt_set_forcing that
need no GPU."""
import ctypes
import dataclasses

import numpy as np
import pytest

from harness import FORCING_CODES, ONX, build_oracle, configs, interior
from oracle.oracle import FORCING_FLUX, FORCING_NONE, FORCING_RELAX


def _random_forcing(kind, seed, scale=1e-3):
    def forcing(m):
        P = tuple(m.n[a] + 2 * ONX for a in (0, 1, 3, 4, 5))
        rng = np.random.default_rng(seed)
        return kind, np.asfortranarray(rng.uniform(0.0, scale, size=P))
    return forcing


def _bottom(n):
    sl = list(interior(n))
    sl[2] = ONX
    return tuple(sl)


def _forced(kind, seed=3, n=(6, 5, 6, 4, 4, 6)):
    return dataclasses.replace(configs.shear_mini(n=n), forcing=_random_forcing(kind, seed))


def _plane5(F, n):
    """interior of a padded 5D field, shaped like the z = 1 plane of E"""
    f = F[ONX:ONX + n[0], ONX:ONX + n[1], ONX:ONX + n[3], ONX:ONX + n[4], ONX:ONX + n[5]]
    return f


def test_flux_forcing_updates_the_bottom_plane_only():
    exp = _forced("flux")
    o = build_oracle(exp)
    E0 = o.E.copy()
    _, F = exp.forcing(o)
    o.apply_forcing()
    dz = o.grid["z"]["dt"][ONX]
    bot = _bottom(exp.n)
    want = E0[bot] + o.dt * _plane5(F, exp.n) / dz     # lee1.f90:206, same operation order
    assert np.array_equal(o.E[bot], want)
    rest = o.E.copy()
    rest[bot] = E0[bot]
    assert np.array_equal(rest, E0)


def test_relax_forcing_formula_fixed_point_and_upward_faces():
    exp = _forced("relax")
    o = build_oracle(exp)
    _, F = exp.forcing(o)
    bot = _bottom(exp.n)
    G = _plane5(F, exp.n)
    E0 = o.E.copy()
    w = o.zdot[bot]
    assert (w > 0).any() and (w < 0).any()             # both signs present in the shear case
    o.apply_forcing()
    got = o.E[bot]
    want = E0[bot] - o.dt * np.where(0.0 > w, 0.0, w) * (E0[bot] - G) / o.grid["z"]["dt"][ONX]
    assert np.array_equal(got, want)                   # critical_gm1.f90:132-133
    assert np.array_equal(got[w <= 0], E0[bot][w <= 0])
    # E = E_gm is a fixed point
    o.E[bot] = G
    o.apply_forcing()
    assert np.array_equal(o.E[bot], G)


def test_step_is_forcing_then_integrate():
    exp = _forced("flux")
    a, b = build_oracle(exp), build_oracle(exp)
    a.integrate(1)
    b.apply_forcing()
    b.lib.orc_integrate(b.s)
    assert np.array_equal(a.E, b.E)
    # and switching it off gives the unforced step
    c, d = build_oracle(exp), build_oracle(configs.shear_mini(n=exp.n))
    c.set_forcing(FORCING_NONE)
    c.integrate(2)
    d.integrate(2)
    assert np.array_equal(c.E, d.E)


def test_oracle_rejects_bad_forcing():
    o = build_oracle(configs.shear_mini())
    with pytest.raises(ValueError):
        o.set_forcing(FORCING_FLUX, np.zeros((3, 3, 3, 3, 3)))
    with pytest.raises(ValueError):
        o.set_forcing(7, None)
    with pytest.raises(ValueError):
        o.set_forcing(FORCING_RELAX, None)


def test_lee_wave_flux_field():
    """flux_lee is positive exactly where f0^2 < om_lee^2 < N^2 at the
    bottom (lee1.f90:117) and zero in the first m ghost plane (:108)."""
    exp = configs.lee_wave_flux(fac=1)
    o = build_oracle(exp)
    kind, F = exp.forcing(o)
    assert kind == "flux" and np.isfinite(F).all() and (F >= 0).all()
    kt = o.grid["k"]["t"]
    U1, N1 = o.U[ONX, ONX, ONX], o.Nsqr[ONX, ONX, ONX]
    om2 = (kt * U1) ** 2
    band = (om2 > exp.f0 ** 2) & (om2 < N1)
    assert band.any() and not band.all()
    assert not F[:, :, ~band, :, :].any()
    assert F[ONX, ONX, band, ONX, 1:].max() > 0
    assert not F[:, :, :, :, 0].any()
    assert FORCING_CODES[kind] == FORCING_FLUX


def test_critical_gm_relax_field_and_column():
    """E_gm is positive and finite on the bottom plane; a forced column with
    no initial energy gains energy only through the bottom."""
    exp = configs.critical_gm_relax(fac=0.5)
    o = build_oracle(exp)
    kind, F = exp.forcing(o)
    assert kind == "relax" and np.isfinite(F).all() and (F > 0).all()
    assert not o.E.any()
    o.integrate(4)
    sl = interior(exp.n)
    assert o.E[sl].max() > 0
    # a step reaches at most two cells (the superbee stencil), so after 4
    # steps nothing lies above z index 8
    assert not o.E[sl][:, :, 9:].any()


def test_set_forcing_argument_checks_without_gpu():
    import __graft_entry__ as g
    g.build_library()
    from raytracer_3d_gb300 import _lib
    lib = _lib.load()
    assert lib.rt_set_forcing(None, _lib.RT_FORCING_FLUX, None) == -1
    assert lib.rt_set_forcing(ctypes.c_void_p(0), _lib.RT_FORCING_NONE, None) == -1
