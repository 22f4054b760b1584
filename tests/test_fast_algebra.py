"""The fast binary64 schedule's algebra (raytracer_3d_gb300/csrc/rt_fast.cu,
rt_fast.cuh) restated in numpy and held against the oracle on the CPU:
the upwind flux F = v*E_up + h*psi with the exactly selected superbee slope
psi and h = |v|/2*(1 - |v dt/d|), the clamped face-0 flux v*E(0), and the
regrouped update E*mu + sum_a dt/d_a*(F_l - F_r) with mu = 1 - dt*lambda.
One step from the oracle's state stays within the fast form's bound of
1e-12 relative L-infinity of the reference's division form
(superbee_fluxes.f90:19-30, integrate.f90:102-268).  No GPU: this pins the
rewritten arithmetic itself; the GPU tests pin the kernels to it."""
import numpy as np
import pytest

from harness import ONX, build_oracle, configs, interior

VEL = ("xdot", "ydot", "zdot", "kdot", "ldot", "mdot")
TOL = 1e-12


def _fill_ghosts(E, n, upper, lower):
    """the boundary order of integrate.f90:14-94 with the serial reflection
    (parallel_mpi.f90:839, :869): z walls with the m index reversed, then
    edge copies on the open sides"""
    E = E.copy()
    nz, nm = n[2], n[5]
    msl = slice(ONX, ONX + nm)
    zaxis = [slice(None)] * 6
    if n[2] > 1:
        for i in (1, 2):
            if upper:   # ghost nz+i <- nz-i+1 at nm+1-m
                g, s = nz + i + ONX - 1, nz - i + 1 + ONX - 1
                src = E[:, :, s, :, :, msl][..., ::-1]
                E[:, :, g, :, :, msl] = src
            if lower:   # ghost 1-i <- i at nm+1-m
                g, s = 1 - i + ONX - 1, i + ONX - 1
                src = E[:, :, s, :, :, msl][..., ::-1]
                E[:, :, g, :, :, msl] = src
    for a in range(6):
        if n[a] <= 1:
            continue
        lo, hi = ONX, ONX + n[a] - 1
        for i in (1, 2):
            sl_g, sl_s = list(zaxis), list(zaxis)
            if not (a == 2 and upper):
                sl_g[a], sl_s[a] = hi + i, hi
                E[tuple(sl_g)] = E[tuple(sl_s)]
            if not (a == 2 and lower):
                sl_g, sl_s = list(zaxis), list(zaxis)
                sl_g[a], sl_s[a] = lo - i, lo
                E[tuple(sl_g)] = E[tuple(sl_s)]
    return E


def _superbee_slope(Rj, up):
    """phi(up/Rj)*Rj selected among Rj, up and their doubles (exact)"""
    s = np.where(np.signbit(Rj), -1.0, 1.0)
    a = np.abs(Rj)
    t = s * up
    lo, hi = np.minimum(a, t), np.maximum(a, t)
    m = np.where(t > 0, np.minimum(2.0 * lo, hi), 0.0)
    return s * m


def _take(E, a, lo, hi):
    sl = [slice(ONX, -ONX)] * 6
    sl[a] = slice(lo, hi)
    return E[tuple(sl)]


def fast_step(o, exp):
    n, dt = exp.n, o.dt
    E = _fill_ghosts(o.E, n, exp.upper, exp.lower)
    acc = np.zeros(n)
    mu = np.ones(n)
    sl_int = interior(n)
    for c, lam in enumerate(("lambda_x", "lambda_y", "lambda_z")):
        if n[c] > 1:
            mu = mu - dt * getattr(o, lam)[sl_int]
    for a in range(6):
        if n[a] <= 1:
            continue
        na = n[a]
        # faces f = 0..na (Fortran), the face between cells f and f+1
        Em1 = _take(E, a, ONX - 2, ONX + na - 1)     # E(f-1)
        E0 = _take(E, a, ONX - 1, ONX + na)          # E(f)
        Ep1 = _take(E, a, ONX, ONX + na + 1)         # E(f+1)
        Ep2 = _take(E, a, ONX + 1, ONX + na + 2)     # E(f+2)
        v = _take(getattr(o, VEL[a]), a, ONX - 1, ONX + na)
        shp = [1] * 6
        shp[a] = na + 1
        d = o.grid["xyzklm"[a]]["dt"][ONX - 1:ONX + na].reshape(shp)   # d(f), f = 0..na
        pos = v > 0
        Rj = Ep1 - E0
        up = np.where(pos, E0, Ep2) - np.where(pos, Em1, Ep1)
        h = 0.5 * np.abs(v) * (1.0 - np.abs(v * dt / d))
        F = h * _superbee_slope(Rj, up) + v * np.where(pos, E0, Ep1)
        if not (a == 2 and exp.lower):
            # face 0 with the edge copied into the ghosts: v*E(0)
            sl0 = [slice(None)] * 6
            sl0[a] = slice(0, 1)
            F[tuple(sl0)] = v[tuple(sl0)] * _take(E, a, ONX, ONX + 1)
        sl_l, sl_r = [slice(None)] * 6, [slice(None)] * 6
        sl_l[a], sl_r[a] = slice(0, na), slice(1, na + 1)
        shc = [1] * 6
        shc[a] = na
        cdt = dt / o.grid["xyzklm"[a]]["dt"][ONX:ONX + na].reshape(shc)
        acc = acc + cdt * (F[tuple(sl_l)] - F[tuple(sl_r)])
    return o.E[sl_int] * mu + acc


CASES = {
    "shear_reflecting": lambda: configs.shear_mini(),
    "shear_open": lambda: configs.shear_mini(upper=False, lower=False),
    "shear_mixed_neg": lambda: configs.shear_mini(upper=True, lower=False, sign_of_omega_i=-1.0),
    "ragged": lambda: configs.shear_mini(n=(7, 3, 5, 2, 6, 4)),
    "stretched": lambda: configs.stretched_mini(),
    "column_1d": lambda: configs.column_1d(fac=1),
}


@pytest.mark.parametrize("name", list(CASES))
def test_fast_algebra_within_bound_of_oracle(name):
    exp = CASES[name]()
    o = build_oracle(exp)
    try:
        for step in range(3):
            got = fast_step(o, exp)
            o.integrate(1)
            ref = o.E[interior(exp.n)]
            scale = np.max(np.abs(ref))
            err = np.max(np.abs(got - ref)) / scale
            assert err <= TOL, (step, err)
    finally:
        o.close()
