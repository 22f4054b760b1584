"""Known-answer tests that pin the CPU oracle to the mathematics of the
reference scheme (superbee_fluxes.f90, integrate.f90, diagnose.f90,
calc_grid.f90, calc_parameter.f90).  The reference ships no tests or golden
data, so these are the oracle's anchor."""
import math

import numpy as np
import pytest

from harness import ONX, build_oracle, configs, interior
from oracle.oracle import Oracle
from raytracer_3d_gb300.grid import calc_grid


def superbee_phi(r):
    """superbee limiter, superbee_fluxes.f90:10"""
    return max(0.0, max(min(1.0, 2.0 * r), min(2.0, r)))


def line_oracle(nx, u0, dx, dt, E_line):
    """1D x-advection: nk = 1 with k_fixed = 0 makes the analytic velocity
    of calc_parameter.f90:98 equal to U, so faces 1..nx carry u0 and face 0
    keeps the allocation value 0."""
    n = (nx, 1, 1, 1, 1, 1)
    o = Oracle(n)
    o.set_spacings([np.full(nx, dx), [1.0], [1.0], [1.0], [1.0], [1.0]])
    o.set_scalars(dt, 1e-4, 1.0, False, False, (0.0, 0.0, 1e-2))
    assert o.calc_grid() == 0
    o.Nsqr[:] = 1e-6
    o.U[:] = u0
    o.V[:] = 0.0
    o.calc_parameter()
    o.E[ONX:ONX + nx, ONX, ONX, ONX, ONX, ONX] = E_line
    return o


@pytest.mark.parametrize("r", [-1.0, 0.0, 0.25, 0.5, 1.0, 1.5, 2.0, 3.0])
def test_limiter_table(r):
    # E = (0, r, r+1, ...): at face 2 (between cells 2 and 3) with v>0:
    # Rjm = E(2)-E(1) = r, Rj = E(3)-E(2) = 1, Cr = Rjm/Rj = r
    nx, u0, dx, dt = 6, 0.5, 100.0, 60.0
    E = np.array([0.0, r, r + 1.0, r + 2.0, r + 2.0, r + 2.0])
    o = line_oracle(nx, u0, dx, dt, E)
    o.integrate(1)
    f = 2
    flux = o.flux_x[f + ONX - 1, ONX, ONX, ONX, ONX, ONX]
    E2, E3 = E[f - 1], E[f]
    Rj = E3 - E2
    uCFL = abs(u0 * dt / dx)
    phi = superbee_phi(r)
    expect = u0 * (E3 + E2) * 0.5 - abs(u0) * ((1.0 - phi) + uCFL * phi) * Rj * 0.5
    assert flux == pytest.approx(expect, rel=1e-15, abs=1e-15)
    # recover phi from the flux
    phi_back = ((u0 * (E3 + E2) * 0.5 - flux) * 2 / (abs(u0) * Rj) - 1.0) / (uCFL - 1.0)
    assert phi_back == pytest.approx(phi, abs=1e-12)


def test_cfl_one_is_exact_shift():
    # uCFL = 1: the superbee flux reduces to the upwind flux v*E_i and one
    # step shifts E by exactly one cell
    nx, u0, dx = 12, 0.25, 1000.0
    dt = dx / u0
    rng = np.random.default_rng(0)
    E = np.concatenate([np.zeros(3), rng.uniform(0.5, 1.5, nx - 6), np.zeros(3)])
    o = line_oracle(nx, u0, dx, dt, E)
    o.integrate(1)
    new = o.E[ONX:ONX + nx, ONX, ONX, ONX, ONX, ONX]
    np.testing.assert_allclose(new[1:], E[:-1], rtol=0, atol=1e-15)


def test_zero_gradient_has_no_diffusive_flux():
    nx, u0, dx, dt = 8, 0.3, 500.0, 100.0
    E = np.full(nx, 2.5)
    o = line_oracle(nx, u0, dx, dt, E)
    o.integrate(1)
    flux = o.flux_x[ONX:ONX + nx, ONX, ONX, ONX, ONX, ONX]   # faces 1..nx
    assert np.all(flux == u0 * 2.5)


def independent_line_step(E, u0, dx, dt):
    """Pure-Python restatement of one x-step of the scheme on an open line
    (face 0 velocity 0 as left by the collapsed-pair branch)."""
    nx = len(E)
    G = [E[0], E[0]] + list(E) + [E[-1], E[-1]]   # ghosts, integrate.f90:24-33
    vel = [0.0] + [u0] * nx                         # faces 0..nx
    flux = []
    for f in range(0, nx + 1):
        v = vel[f]
        g = f + 1  # position of cell f (Fortran) in G, cell 1 at G[2]
        uCFL = abs(v * dt / dx)
        Rjp = G[g + 2] - G[g + 1]
        Rj = G[g + 1] - G[g]
        Rjm = G[g] - G[g - 1]
        if Rj != 0.0:
            Cr = Rjm / Rj if v > 0 else Rjp / Rj
        else:
            Cr = (Rjm if v > 0 else Rjp) * float(np.float32(1e20))
        Cr = superbee_phi(Cr)
        flux.append(v * (G[g + 1] + G[g]) * 0.5 - abs(v) * ((1.0 - Cr) + uCFL * Cr) * Rj * 0.5)
    out = []
    for i in range(1, nx + 1):
        dE = 0.0 - (flux[i] - flux[i - 1]) / dx
        dE = dE - 0.0
        out.append(E[i - 1] + dt * dE)
    return np.array(out)


def test_line_matches_independent_restatement():
    nx, u0, dx, dt = 16, 0.4, 250.0, 300.0
    rng = np.random.default_rng(3)
    E = rng.uniform(0.0, 1.0, nx)
    o = line_oracle(nx, u0, dx, dt, E)
    ref = E.copy()
    for _ in range(4):
        o.integrate(1)
        ref = independent_line_step(ref, u0, dx, dt)
    got = o.E[ONX:ONX + nx, ONX, ONX, ONX, ONX, ONX]
    assert np.array_equal(got, ref)


def test_grid_restatements_agree():
    e = configs.shear_mini()
    o = build_oracle(e)
    g = calc_grid(e.n, e.d_interior, e.fixed)
    for ax in ("x", "y", "z", "k", "l", "m"):
        for key in ("t", "u", "dt", "du"):
            assert np.array_equal(o.grid[ax][key], g[ax][key]), (ax, key)


def test_dispersion_relation():
    e = configs.shear_mini()
    o = build_oracle(e)
    kt, lt, mt = (o.grid[a]["t"] for a in ("k", "l", "m"))
    K = kt[None, None, None, :, None, None]
    L = lt[None, None, None, None, :, None]
    M = mt[None, None, None, None, None, :]
    N2 = o.Nsqr[:, :, :, None, None, None]
    kh2 = L * L + K * K
    om = np.sqrt((N2 * kh2 + (e.f0 * e.f0) * (M * M)) / (M * M + kh2))
    assert np.array_equal(o.omega_i, om)
    ome = (om + K * o.U[..., None, None, None]) + L * o.V[..., None, None, None]
    assert np.array_equal(o.omega_e, ome)
    # frequencies lie between f and N
    sl = interior(e.n)
    assert np.all(o.omega_i[sl] >= e.f0 * (1 - 1e-12))
    assert np.all(o.omega_i[sl] <= np.sqrt(o.Nsqr.max()) * (1 + 1e-12))


def _zdot_error(nm):
    e = configs.shear_mini(n=(4, 4, 4, 4, 4, nm))
    o = build_oracle(e)
    kt, lt, mt = (o.grid[a]["t"] for a in ("k", "l", "m"))
    sl = interior(e.n)
    N2 = o.Nsqr[sl[:3]][..., None, None, None]
    K = kt[ONX:-ONX][None, None, None, :, None, None]
    L = lt[ONX:-ONX][None, None, None, None, :, None]
    M = mt[ONX:-ONX][None, None, None, None, None, :]
    kh2 = K * K + L * L
    om = np.sqrt((N2 * kh2 + e.f0 ** 2 * M * M) / (M * M + kh2))
    dom_dm = (e.f0 ** 2 - N2) * kh2 * M / (om * (M * M + kh2) ** 2)   # d omega / dm
    got = o.zdot[sl]
    keep = np.broadcast_to(np.abs(M) >= 0.02, got.shape)
    return float(np.max(np.abs(got - dom_dm)[keep] / np.abs(dom_dm)[keep]))


def test_velocities_are_group_velocities():
    # zdot (calc_parameter.f90:198-200) converges to d omega/dm at second
    # order as the m grid is refined
    e32, e64 = _zdot_error(32), _zdot_error(64)
    assert e64 < 0.02
    assert e32 / e64 > 3.0


def test_budget_residual_vanishes():
    e = configs.shear_mini()
    o = build_oracle(e)
    for _ in range(3):
        o.integrate(1)
        b = o.diagnose()
        scale = abs(b["eint"]) + abs(b["mflint"]) + sum(abs(b[k]) for k in b if k.startswith("bfl"))
        assert abs(b["residual"]) <= 1e-13 * scale


def test_energy_change_equals_budget():
    e = configs.shear_mini(upper=False, lower=False)
    o = build_oracle(e)
    sl = interior(e.n)
    vol = np.ones(e.n)
    for a in range(6):
        shp = [1] * 6
        shp[a] = e.n[a]
        vol = vol * o.grid["xyzklm"[a]]["dt"][ONX:ONX + e.n[a]].reshape(shp)
    tot0 = float(np.sum(o.E[sl] * vol))
    o.integrate(1)
    b = o.diagnose()
    tot1 = float(np.sum(o.E[sl] * vol))
    assert tot1 - tot0 == pytest.approx(o.dt * b["eint"], rel=1e-10)


def test_positivity_at_cfl_04():
    e = configs.shear_mini(n=(8, 6, 8, 6, 6, 8))
    o = build_oracle(e)
    for _ in range(10):
        o.integrate(1)
    assert np.min(o.E[interior(e.n)]) >= 0.0


def test_column_1d_reduces_to_z_m():
    # the reference's 1D setup (test1D.f90): only z and m are active, the
    # x velocity follows the analytic branch of calc_parameter.f90:98 and
    # kdot stays 0
    e = configs.column_1d()
    o = build_oracle(e)
    sl = interior(e.n)
    assert np.all(o.kdot == 0.0)
    assert np.max(np.abs(o.xdot[sl])) > 0
    E0 = o.E[sl].copy()
    o.integrate(2)
    assert np.all(o.flux_x == 0.0) and np.all(o.flux_k == 0.0)
    assert not np.array_equal(o.E[sl], E0)


def test_single_precision_literals():
    assert float(np.float32(1e20)) == 1.0000000200408773e20
    assert float(np.float32(np.pi)) == 3.1415927410125732
    assert float(np.float32(1e-12)) == 9.999999960041972e-13


def test_ensemble_grids_pass_reference_checks():
    # every dims combination of the batched / served workloads builds a grid
    # that the reference's calc_grid accepts
    import itertools
    from raytracer_3d_gb300.configs import SPATIAL_DIMS, SPECTRAL_DIMS, ensemble_member
    rng = np.random.default_rng(0)
    for nz, nm in itertools.product(SPATIAL_DIMS + (4, 6), SPECTRAL_DIMS + (4, 6)):
        e = ensemble_member(rng, spatial=(nz,), spectral=(nm,))
        calc_grid(e.n, e.d_interior, e.fixed)
