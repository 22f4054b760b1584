"""Host-side grid construction: calc_grid (for_src/calc_grid.f90:4-295) on one
rank.

This is setup work of the host driver, not of the GPU path: it turns the
interior grid spacings chosen by an experiment (set_grid) into the padded
1D arrays xt, xu, dxt, dxu, ... that rt_set_grid uploads.  Arrays are padded
by ONX = 2 on both sides; Fortran index f sits at position f + 1.
"""
import numpy as np

ONX = 2
AXES = ("x", "y", "z", "k", "l", "m")


class GridError(ValueError):
    pass


def u_centered_grid(dyt):
    """u_centered_grid, calc_grid.f90:300-322 (n = len(dyt), 0-based)."""
    n = len(dyt)
    yu = np.zeros(n)
    yt = np.zeros(n)
    dyu = np.zeros(n)
    yu[0] = 0.0
    for i in range(1, n):
        yu[i] = yu[i - 1] + dyt[i]
    yt[0] = yu[0] - dyt[0] * 0.5
    for i in range(1, n):
        yt[i] = 2 * yu[i - 1] - yt[i - 1]
    for i in range(n - 1):
        dyu[i] = yt[i + 1] - yt[i]
    dyu[n - 1] = 2 * dyt[n - 1] - dyu[max(1, n - 1) - 1]
    return dyu, yt, yu


def calc_grid(n, d_interior, fixed=(0.0, 0.0, 0.0)):
    """Build padded grids for the six axes.

    n          -- (nx, ny, nz, nk, nl, nm)
    d_interior -- six arrays of interior spacings (length n_a)
    fixed      -- (k_fixed, l_fixed, m_fixed), used when that axis has n=1
    Returns {axis: {"t","u","dt","du"}}; raises GridError on the checks of
    calc_grid.f90:260-293.
    """
    out = {}
    for a, ax in enumerate(AXES):
        na = n[a]
        d = np.zeros(na + 2 * ONX)
        d[ONX:ONX + na] = np.asarray(d_interior[a], dtype=np.float64)
        for i in range(1, ONX + 1):                       # calc_grid.f90:104-111
            d[na + i + ONX - 1] = d[na + ONX - 1]
            d[1 - i + ONX - 1] = d[ONX]
        du, t, u = u_centered_grid(d)
        P = lambda f: f + ONX - 1  # noqa: E731
        if ax in ("x", "y"):                              # :115, :124
            sh = du[P(1)]
            t = t - sh
            u = u - sh
        elif ax == "z":                                   # :133
            sh = u[P(na)]
            t = t - sh
            u = u - sh
        else:                                             # :142-146 etc.
            if na > 1:
                sh = u[P(na // 2)]
                t = t - sh
                u = u - sh
            else:
                fx = fixed[a - 3]
                t = np.full_like(t, fx)
                u = np.full_like(u, fx)
        out[ax] = {"t": t, "u": u, "dt": d, "du": du}
    # monotonicity checks, calc_grid.f90:260-293
    P = lambda f: f + ONX - 1  # noqa: E731
    for ax, hi, name in (("z", n[2], "dzu/dzt"), ("m", n[5] // 2, "dmu/dmt"), ("l", n[4] // 2, "dlu/dlt")):
        du, d = out[ax]["du"], out[ax]["dt"]
        for i in range(2, hi + 1):
            if du[P(i)] - du[P(i - 1)] > 1e-12 or d[P(i)] - d[P(i - 1)] > 1e-12:
                raise GridError(" Error in %s grid setup, %s do not decrease monotonically at i=%d"
                                % (ax, name, i))
    return out
