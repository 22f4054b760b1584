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


# ---------------------------------------------------------------------------
# stretched grids of the reference's configurations (for_config/gm1.f90:33-49,
# brava.f90:32-58): the spacing falls as 1 - 0.8*x**1.5 along a half axis and
# its scale d0 is the root of a closure condition, found by bisection.  The
# reference evaluates these in default real, so they are computed in binary32
# here too and widened to binary64 at the end.
# ---------------------------------------------------------------------------
F32 = np.float32


def bisect(f, lo, hi, tol, max_halvings=40):
    """Root of the increasing-or-decreasing function f on [lo, hi] by the
    bisection method in binary32 arithmetic.  The bracket is halved until
    its nominal width (halved exactly each time, so that it keeps shrinking
    below the binary32 spacing of the root) is below tol; returns the
    bracket end at which f <= 0.  Raises GridError when [lo, hi] does not
    bracket a sign change or when max_halvings are not enough."""
    lo, hi = F32(lo), F32(hi)
    flo, fhi = f(lo), f(hi)
    if not (flo < 0) ^ (fhi < 0):
        raise GridError("bisection: the interval [%g, %g] does not bracket a root" % (lo, hi))
    below, above = (lo, hi) if flo < 0 else (hi, lo)     # f(below) < 0 <= f(above)
    width = F32(above - below)
    for _ in range(max_halvings):
        width = F32(width * F32(0.5))
        mid = F32(below + width)
        fm = f(mid)
        if fm <= 0:
            below = mid
        if abs(width) < tol or fm == 0:
            return below
    raise GridError("bisection: no convergence after %d halvings" % max_halvings)


def stretched_half(d0, start, count):
    """Positions p(0..count) and spacings d(1..count) (index 0 unused) of
    the stretched half axis: p(0) = start, d(i) = d0*(1 - x(i)**1.5*0.8)
    with x(i) = (i-1)/(count-1), p(i) = p(i-1) + d(i), in binary32
    (gm1.f90 mgrid/lgrid, brava.f90 zgrid)."""
    if count < 2:
        raise GridError("a stretched half axis needs at least 2 cells")
    p = np.zeros(count + 1, dtype=F32)
    d = np.zeros(count + 1, dtype=F32)
    p[0] = F32(start)
    den = F32(F32(count) - F32(1.0))
    for i in range(1, count + 1):
        x = F32(F32(F32(i) - F32(1.0)) / den)
        d[i] = F32(F32(d0) * F32(F32(1) - F32(F32(x ** F32(1.5)) * F32(0.8))))
        p[i] = F32(p[i - 1] + d[i])
    return p, d


def symmetric_stretched(n, start, lo=None, hi=None, tol=None):
    """Spacings of a spectral axis of n (even, >= 4) cells refined towards
    zero and mirrored about it (gm1.f90:45-47): d0 makes the centre fall on
    the middle face, p(n/2) + d(n/2) = 0, starting from p(0) = start.  The
    bisection tolerance defaults to 1e-8 of the half span (the reference's
    1e-8 for its span of 1)."""
    if n < 4 or n % 2:
        raise GridError("symmetric stretched axis needs an even n >= 4, got %d" % n)
    half = n // 2

    def closure(d0):
        p, d = stretched_half(d0, start, half)
        return F32(p[half] + d[half])

    span = abs(float(start))
    tol = 1e-8 * span if tol is None else tol
    lo = span / (100.0 * half) if lo is None else lo
    hi = 4.0 * span / half if hi is None else hi
    d0 = bisect(closure, lo, hi, tol)
    _, d = stretched_half(d0, start, half)
    first = d[1:half + 1]
    return np.concatenate([first, first[::-1]]).astype(np.float64)


def bottom_refined(nz, Lz, lo=None, hi=None, tol=1e-8):
    """z spacings of nz cells decreasing upward over a depth Lz (brava.f90
    zgrid / zfunc): z(0) = -Lz - dz0/2 and dz0 makes the last centre fall on
    z = 0, z(nz) + dz(nz)/2 = 0."""
    Lz32 = F32(Lz)

    def positions(dz0):
        return stretched_half(dz0, F32(-Lz32 - F32(F32(dz0) / F32(2))), nz)

    def closure(dz0):
        p, d = positions(dz0)
        return F32(p[nz] + F32(d[nz] / F32(2.0)))

    lo = float(Lz) / nz / 10.0 if lo is None else lo
    hi = float(Lz) if hi is None else hi
    dz0 = bisect(closure, lo, hi, tol)
    _, d = positions(dz0)
    return d[1:].astype(np.float64)


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
