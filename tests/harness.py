"""Shared test helpers: build the oracle and the GPU model from one
experiment description, and compare arrays on the ranges the path uses."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle.oracle import FORCING_FLUX, FORCING_RELAX, Oracle  # noqa: E402
from raytracer_3d_gb300 import configs  # noqa: E402
from raytracer_3d_gb300.grid import ONX  # noqa: E402


FORCING_CODES = {"flux": FORCING_FLUX, "relax": FORCING_RELAX}


def build_oracle(exp, threads=False):
    """The reference setup order (main.f90:36-47) on the oracle."""
    o = Oracle(exp.n, threads=threads)
    o.set_spacings(exp.d_interior)
    dt0 = exp.dt if exp.dt else 1.0
    o.set_scalars(dt0, exp.f0, exp.sign_of_omega_i, exp.upper, exp.lower, exp.fixed)
    rc = o.calc_grid()
    assert rc == 0, "oracle calc_grid check failed (%d)" % rc
    exp.background(o)
    exp.initial(o, np.random.Generator(np.random.PCG64(exp.seed)))
    o.calc_parameter()
    if exp.cfl is not None:
        dt = exp.cfl / o.max_rate()
        o.set_scalars(dt, exp.f0, exp.sign_of_omega_i, exp.upper, exp.lower, exp.fixed)
        o.dt = dt
    else:
        o.dt = exp.dt
    if exp.forcing is not None:
        kind, F = exp.forcing(o)
        o.set_forcing(FORCING_CODES[kind], F)
    return o


def build_point_oracle(exp, dt, threads=True):
    """the per-cell oracle of an experiment: grids and background as in
    build_oracle, dt given (the CFL-defined dt needs whole coefficient
    fields; the caller passes the one the GPU uses, which the coefficient
    parity tests pin on smaller cases)"""
    o = Oracle(exp.n, threads=threads, light=True)
    o.set_spacings(exp.d_interior)
    o.set_scalars(dt, exp.f0, exp.sign_of_omega_i, exp.upper, exp.lower, exp.fixed)
    rc = o.calc_grid()
    assert rc == 0, "oracle calc_grid check failed (%d)" % rc
    exp.background(o)
    o.dt = dt
    return o


def sample_cells(n, count, rng):
    """interior cells (Fortran indices), half of them on a boundary plane of
    a random axis (first or last index) so that faces and z walls are hit"""
    cells = np.stack([rng.integers(1, k + 1, size=count) for k in n], axis=1)
    edge = rng.random(count) < 0.5
    ax = rng.integers(0, 6, size=count)
    hi = rng.random(count) < 0.5
    for q in np.nonzero(edge)[0]:
        cells[q, ax[q]] = n[ax[q]] if hi[q] else 1
    return cells.astype(np.int32)


def interior(n):
    return tuple(slice(ONX, ONX + k) for k in n)


def face_range(n, a):
    """faces 0..n along axis a, interior elsewhere (padded positions)."""
    sl = list(interior(n))
    sl[a] = slice(ONX - 1, ONX + n[a])
    return tuple(sl)


def max_rel(a, b):
    """max |a-b| / max |b| (0 when both vanish)."""
    den = float(np.max(np.abs(b)))
    num = float(np.max(np.abs(a - b)))
    return num / den if den > 0 else num


def vol_weights(model):
    """the six 1D cell widths of a model's interior (binary64)"""
    return [model.grid["xyzklm"[a]]["dt"][ONX:ONX + model.n[a]] for a in range(6)]


def energy_sum(E, widths):
    """total energy sum(E * vol) of an interior 6D array, vol the product of
    the cell widths, accumulated one m plane at a time (no full-size
    temporaries at 32^6)"""
    v5 = np.ones([len(w) for w in widths[:5]])
    for a in range(5):
        shp = [1] * 5
        shp[a] = len(widths[a])
        v5 = v5 * widths[a].reshape(shp)
    tot = 0.0
    for m in range(E.shape[5]):
        tot += float(np.sum(np.asarray(E[..., m], dtype=np.float64) * v5)) * float(widths[5][m])
    return tot


def error_norms(got, ref):
    """relative L2 and L-infinity (relative to max |ref|) of got - ref,
    accumulated one m plane at a time"""
    num2 = den2 = 0.0
    dmax = rmax = 0.0
    for m in range(ref.shape[5]):
        r = np.asarray(ref[..., m], dtype=np.float64)
        d = np.asarray(got[..., m], dtype=np.float64) - r
        num2 += float(np.sum(d * d))
        den2 += float(np.sum(r * r))
        dmax = max(dmax, float(np.max(np.abs(d))))
        rmax = max(rmax, float(np.max(np.abs(r))))
    return (num2 ** 0.5) / (den2 ** 0.5), dmax / rmax


def rounding_noise_bound(E, widths, steps, sigmas=4.0):
    """drift allowance from the binary32 update's unbiased rounding noise:
    each step rounds every cell to one of its two binary32 neighbours with
    zero mean error and a standard deviation of at most 2^-23/sqrt(6) of the
    cell's value, independently, so the total energy drifts as a random walk
    of relative standard deviation 2^-23/sqrt(6) * sqrt(steps / N_eff), with
    N_eff = (sum E vol)^2 / sum (E vol)^2 the effective number of cells
    carrying the energy.  Returns sigmas of that deviation."""
    v5 = np.ones([len(w) for w in widths[:5]])
    for a in range(5):
        shp = [1] * 5
        shp[a] = len(widths[a])
        v5 = v5 * widths[a].reshape(shp)
    s1 = s2 = 0.0
    for m in range(E.shape[5]):
        ev = np.asarray(E[..., m], dtype=np.float64) * v5 * float(widths[5][m])
        s1 += float(np.sum(ev))
        s2 += float(np.sum(ev * ev))
    n_eff = s1 * s1 / s2
    return sigmas * 2.0 ** -23 / 6 ** 0.5 * (steps / n_eff) ** 0.5
