"""Experiment definitions (the role of for_config/*.f90: set_parameter,
set_grid, set_initial_conditions) for the workloads this package is measured
and tested on.

Each experiment is a plain description; `build_model` turns it into a
`Model` by the reference's setup order (main.f90:36-47).  Inputs are seeded
and synthetic.  Where a workload description and the reference differ the
reference wins: x and y boundaries are the reference's open outflow
(integrate.f90:24-45; it has no periodic mode), spectral grids are centred
on zero as calc_grid.f90:167-169 builds them (the z reflection reverses m,
parallel_mpi.f90:839), and dt comes from a CFL number through the maximum
cell rate (the reference sets dt by hand and only prints the CFL number,
diagnose.f90:295-317).
"""
import math
from dataclasses import dataclass, field
from typing import Callable, Optional, Tuple

import numpy as np

from . import grid
from .grid import ONX
from .model import Model, zeros_padded

# default-real constants of the reference, widened to binary64
PI_F = float(np.float32(np.pi))          # main_module.f90:10


def f32(x):
    """A Fortran default-real literal widened to binary64."""
    return float(np.float32(x))


@dataclass
class Experiment:
    name: str
    n: Tuple[int, int, int, int, int, int]
    d_interior: list
    f0: float
    background: Callable            # (model) -> fills model.Nsqr/U/V (padded)
    initial: Callable               # (model, rng) -> fills model.E
    steps: int
    dt: Optional[float] = None
    cfl: Optional[float] = None
    sign_of_omega_i: float = 1.0
    upper: bool = True
    lower: bool = True
    fixed: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    seed: int = 1234
    meta: dict = field(default_factory=dict)
    # set_forcing of the forced configurations: (model) -> (kind, F) with
    # kind "flux" or "relax" and F the padded 5D field (x,y,k,l,m)
    forcing: Optional[Callable] = None

    @property
    def cells(self):
        return int(np.prod(self.n))


def build_model(exp, precision="fp64", padded=True):
    """set_parameter .. calc_parameter for one experiment; returns a Model
    with the initial state uploaded and dt fixed (from the CFL number when
    the experiment gives one).  padded=False keeps only the interior of the
    state on the host (the serving layer; experiments whose initial
    condition goes through _interior)."""
    m = Model(*exp.n, dt=exp.dt if exp.dt else 1.0, f0=exp.f0, sign_of_omega_i=exp.sign_of_omega_i,
              enable_upper_reflection=exp.upper, enable_lower_reflection=exp.lower,
              precision=precision, k_fixed=exp.fixed[0], l_fixed=exp.fixed[1], m_fixed=exp.fixed[2],
              padded=padded)
    m.calc_grid(exp.d_interior)
    exp.background(m)
    exp.initial(m, np.random.Generator(np.random.PCG64(exp.seed)))
    m.calc_parameter()
    if exp.cfl is not None:
        m.set_dt(exp.cfl / m.max_rate())
    if exp.forcing is not None:
        kind, F = exp.forcing(m)
        m.set_forcing(kind, F)
    m.set_state()
    return m


def _mesh3(m):
    xt, yt, zt = m.grid["x"]["t"], m.grid["y"]["t"], m.grid["z"]["t"]
    return np.meshgrid(xt, yt, zt, indexing="ij")


def _interior(m):
    if not getattr(m, "padded", True):
        return tuple(slice(0, k) for k in m.n)
    return tuple(slice(ONX, ONX + k) for k in m.n)


def _packet(m, rng, center, width_cells, amp, noise):
    """Gaussian packet on the interior (widths in cells of each axis), built
    as the outer product of six 1D Gaussians, plus uniform noise."""
    sl = _interior(m)
    E = np.full((1,) * 6, float(amp))
    for a, ax in enumerate(("x", "y", "z", "k", "l", "m")):
        t = m.grid[ax]["t"][ONX:ONX + m.n[a]]
        if m.n[a] == 1 or center[a] is None:
            g1 = np.ones(m.n[a])
        else:
            d = m.grid[ax]["dt"][ONX:ONX + m.n[a]]
            g1 = np.exp(-0.5 * ((t - center[a]) / (width_cells * d)) ** 2)
        shp = [1] * 6
        shp[a] = m.n[a]
        E = E * g1.reshape(shp)
    if noise:
        E = E + rng.uniform(0.0, noise, size=m.n)
    m.E[sl] = E


# ---------------------------------------------------------------------------
# workload 1: plain FP64 packet, CPU-sized
# ---------------------------------------------------------------------------
def packet_small(n=(8, 8, 16, 16, 16, 16), steps=200, seed=1234, Lx=40e3, Ly=40e3, Lz=4000.0,
                 kmax=2e-3, lmax=2e-3, mmax=5e-2, cfl=0.4):
    """8x8x16 x 16^3, f=1e-4, N(z)=5e-3 exp(z/1000 m) over 4000 m, no mean
    flow, Gaussian packet at mid x,y,z and (k0,l0,m0)=(1e-3,0,1e-2), widths
    2 cells, amplitude 1e-3 plus U(0,1e-8) noise, CFL 0.4."""
    nx, ny, nz, nk, nl, nm = n
    d = [np.full(nx, Lx / nx), np.full(ny, Ly / ny), np.full(nz, Lz / nz),
         np.full(nk, 2 * kmax / nk), np.full(nl, 2 * lmax / nl), np.full(nm, 2 * mmax / nm)]

    def background(m):
        X, Y, Z = _mesh3(m)
        m.Nsqr[:] = (5e-3 * np.exp(Z / 1000.0)) ** 2
        m.U[:] = 0.0
        m.V[:] = 0.0

    def initial(m, rng):
        c = (Lx / 2, Ly / 2, -Lz / 2, 1e-3, 0.0, 1e-2)
        _packet(m, rng, c, 2.0, 1e-3, 1e-8)

    return Experiment("packet_small", tuple(n), d, 1e-4, background, initial, steps, cfl=cfl, seed=seed)


# ---------------------------------------------------------------------------
# workloads 2/3: 32^6 with a mean flow
# ---------------------------------------------------------------------------
def jet_large(n=(32, 32, 32, 32, 32, 32), steps=100, seed=4321, Lx=160e3, Ly=160e3, Lz=4000.0,
              kmax=2e-3, lmax=2e-3, mmax=5e-2, cfl=0.4):
    """32^3 x 32^3, U = 0.1 sin(2 pi y/Ly) exp(z/500) m/s, N and f as the
    small packet, E = seeded log-normal spectrum in (k,l,m) times a uniform
    spatial envelope, CFL 0.4."""
    nx, ny, nz, nk, nl, nm = n
    d = [np.full(nx, Lx / nx), np.full(ny, Ly / ny), np.full(nz, Lz / nz),
         np.full(nk, 2 * kmax / nk), np.full(nl, 2 * lmax / nl), np.full(nm, 2 * mmax / nm)]

    def background(m):
        X, Y, Z = _mesh3(m)
        m.Nsqr[:] = (5e-3 * np.exp(Z / 1000.0)) ** 2
        m.U[:] = 0.1 * np.sin(2 * np.pi * Y / Ly) * np.exp(Z / 500.0)
        m.V[:] = 0.0

    def initial(m, rng):
        spec = np.exp(0.5 * rng.standard_normal(m.n[3:]))
        E = 1e-3 * np.broadcast_to(spec[None, None, None], m.n)
        m.E[_interior(m)] = E

    return Experiment("jet_large", tuple(n), d, 1e-4, background, initial, steps, cfl=cfl, seed=seed)


# ---------------------------------------------------------------------------
# small all-axes case with a fully 3D mean flow (exercises every lambda term)
# ---------------------------------------------------------------------------
def shear_mini(n=(6, 5, 6, 4, 4, 6), steps=3, seed=7, upper=True, lower=True, cfl=0.4,
               sign_of_omega_i=1.0):
    nx, ny, nz, nk, nl, nm = n
    Lx, Ly, Lz = 30e3, 25e3, 3000.0
    d = [np.full(nx, Lx / nx), np.full(ny, Ly / ny), np.full(nz, Lz / nz),
         np.full(nk, 4e-3 / nk), np.full(nl, 4e-3 / nl), np.full(nm, 0.1 / nm)]

    def background(m):
        X, Y, Z = _mesh3(m)
        m.Nsqr[:] = (4e-3 * np.exp(Z / 1500.0)) ** 2 * (1 + 0.1 * np.cos(2 * np.pi * X / Lx))
        m.U[:] = 0.15 * np.sin(2 * np.pi * Y / Ly) * np.exp(Z / 800.0) + 0.02 * np.cos(2 * np.pi * X / Lx)
        m.V[:] = 0.05 * np.cos(2 * np.pi * X / Lx) * np.exp(Z / 1200.0) + 0.01 * np.sin(2 * np.pi * Y / Ly)

    def initial(m, rng):
        c = (Lx / 3, Ly / 2, -Lz / 2, 5e-4, -5e-4, 1.5e-2)
        _packet(m, rng, c, 1.5, 1e-3, 1e-6)

    return Experiment("shear_mini", tuple(n), d, 1.2e-4, background, initial, steps, cfl=cfl, seed=seed,
                      upper=upper, lower=lower, sign_of_omega_i=sign_of_omega_i)


# ---------------------------------------------------------------------------
# the reference's 1D / 2D test setups (for_config/test1D.f90, test2D.f90):
# collapsed axes and the analytic-velocity branch
# ---------------------------------------------------------------------------
def column_1d(fac=2, steps=3):
    """test1D: nz=20*fac, nm=60*fac, other axes 1, k_fixed=1e-3 (test1D.f90:3-78)."""
    nz, nm = int(20 * fac), int(60 * fac)
    f0 = f32(1e-4)
    Lx = Ly = Lz = f32(2000.0)
    n = (1, 1, nz, 1, 1, nm)
    d = [np.full(1, Lx / 1), np.full(1, Ly / 1), np.full(nz, Lz / nz),
         np.full(1, PI_F / Lx), np.full(1, PI_F / Ly), np.full(nm, PI_F / Lz / 4.0)]

    def background(m):
        X, Y, Z = _mesh3(m)
        m.U[:] = 0.50 * (1 + np.tanh((Z + 750) / 150)) / 2.0
        m.Nsqr[:] = (30 * f0) ** 2
        m.V[:] = 0.0

    def initial(m, rng):
        mt = m.grid["m"]["t"]
        zt = m.grid["z"]["t"]
        dmt1 = m.grid["m"]["dt"][ONX]
        for mm in range(1, nm + 1):
            if mt[mm + 1] < 0:
                for kk in range(1, nz + 1):
                    m.E[ONX, ONX, kk + 1, ONX, ONX, mm + 1] = 1.0 + np.sin(
                        mt[mm + 1] * 2 * PI_F / (nm * dmt1 / 2 / 6.0)) * np.sin(zt[kk + 1] * 2 * PI_F / (Lz / 6.0))

    return Experiment("column_1d", n, d, f0, background, initial, steps, dt=5.0 / fac,
                      fixed=(f32(1e-3), 0.0, 0.0))


def section_2d(fac=1, steps=3):
    """test2D: ny=10*fac, nz=20*fac, nl=nm=60*fac, nx=nk=1 (test2D.f90:85-167)."""
    ny, nz, nl, nm = int(10 * fac), int(20 * fac), int(60 * fac), int(60 * fac)
    f0 = f32(1e-4)
    Lz, Ly, Lx = f32(2000.0), f32(20000.0), f32(20000.0)
    n = (1, ny, nz, 1, nl, nm)
    d = [np.full(1, Lx / 1), np.full(ny, Ly / ny), np.full(nz, Lz / nz),
         np.full(1, PI_F / Lx), np.full(nl, 10 * PI_F / Ly), np.full(nm, PI_F / Lz / 4.0)]

    def background(m):
        X, Y, Z = _mesh3(m)
        m.U[:] = f32(0.2) * (1 + np.tanh((Z + 750) / 150)) / 2.0 * np.exp(-(Y - Ly / 2.0) ** 2 / 5000 ** 2)
        m.Nsqr[:] = (30 * f0) ** 2
        m.V[:] = 0.0

    def initial(m, rng):
        mt = m.grid["m"]["t"]
        neg = (mt < 0).astype(np.float64)
        m.E[:] = neg.reshape((1, 1, 1, 1, 1, -1)) * np.ones(m.E.shape)

    return Experiment("section_2d", n, d, f0, background, initial, steps, dt=40.0 / fac,
                      fixed=(f32(1e-3), 0.0, 0.0))


# ---------------------------------------------------------------------------
# the reference's forced configurations (for_config/lee1.f90,
# critical_gm1.f90): a bottom forcing applied before every step
# ---------------------------------------------------------------------------
def _bottom_fill(m, f):
    """U / V ghost planes below z = 1 and above z = nz copy the edge planes
    (lee1.f90:74-85, critical_gm1.f90:70-79)."""
    nz = m.n[2]
    for arr in f:
        for k in range(ONX):
            arr[:, :, k] = arr[:, :, ONX]
            arr[:, :, ONX + nz + k] = arr[:, :, ONX + nz - 1]


def _forcing_mesh(m):
    """kt(l), lt(n), mt(m), dmt(m) on the padded 5D (x,y,k,l,m) shape."""
    P = [m.n[a] + 2 * ONX for a in range(6)]
    kt = m.grid["k"]["t"].reshape(1, 1, P[3], 1, 1)
    lt = m.grid["l"]["t"].reshape(1, 1, 1, P[4], 1)
    mt = m.grid["m"]["t"].reshape(1, 1, 1, 1, P[5])
    dmt = m.grid["m"]["dt"].reshape(1, 1, 1, 1, P[5])
    return P, kt, lt, mt, dmt


def lee_wave_flux(fac=2, steps=3, nz=20):
    """lee1: nz=20, nk=24*fac, nm=26*fac, nx=ny=nl=1; mean flow and N of the
    lee-wave setup and the bottom lee-wave energy flux flux_lee added to the
    z = 1 plane every step (lee1.f90:14-229).  Default-real literals are
    evaluated as the reference does (binary32 where the whole expression is
    default real)."""
    nk, nm = int(24 * fac), int(26 * fac)
    f0 = f32(1e-4)
    Lz, Ly, Lx = f32(2000.0), 240e3, 240e3
    n = (1, 1, nz, nk, 1, nm)
    # lee1.f90:46-51: dkt = 0.004/nk*2 etc. are default-real expressions
    dk = float(np.float32(0.004) / np.float32(nk) * np.float32(2))
    dl = float(np.float32(0.02) / np.float32(nk) * np.float32(2))
    dm = float(np.float32(0.07) / np.float32(nm) * np.float32(2))
    d = [np.full(1, Lx / 1), np.full(1, Ly / 1), np.full(nz, Lz / nz),
         np.full(nk, dk), np.full(1, dl), np.full(nm, dm)]

    def background(m):
        X, Y, Z = _mesh3(m)
        m.U[:] = f32(0.1) + f32(0.10) * (1 + np.tanh((Z + 750) / 150)) / 2.0
        m.Nsqr[:] = np.square(f32(2e-4) + f32(30e-4) * np.exp(Z / 800.0))
        m.V[:] = 0.0
        _bottom_fill(m, (m.U, m.V))

    def initial(m, rng):
        m.E[:] = 0.0

    def forcing(m):
        # lee1.f90:102-132 on the bottom plane k = 1, m from 0 (ms-onx+1)
        P, kt, lt, mt, dmt = _forcing_mesh(m)
        h_rms, nu, k_s = 10.0, f32(0.8), float(np.float32(1) / np.float32(10e3))
        U1 = m.U[:, :, ONX].reshape(P[0], P[1], 1, 1, 1)
        V1 = m.V[:, :, ONX].reshape(P[0], P[1], 1, 1, 1)
        N1 = m.Nsqr[:, :, ONX].reshape(P[0], P[1], 1, 1, 1)
        kh = np.sqrt(kt * kt + lt * lt)
        om = -(kt * U1 + lt * V1)
        om2 = om * om
        ok = (om2 > f0 * f0) & (om2 < N1)
        with np.errstate(divide="ignore", invalid="ignore"):
            m_lee = -kh * np.sqrt(N1 - om2) / np.sqrt(om2 - f0 * f0)
            F_top = h_rms * h_rms * nu / (PI_F * (k_s * k_s)) / np.power(1.0 + (kh / k_s) * (kh / k_s), nu + 1.0)
            freq_fac = 4 * (PI_F * PI_F) * np.sqrt(N1 - om2) * np.sqrt(om2 - f0 * f0) * np.abs(om) / kh
            dd = mt - m_lee
            tw = 2 * dmt
            flux = freq_fac * F_top * np.exp(-(dd * dd) / (tw * tw)) / (2 * dmt * np.sqrt(PI_F))
        ok = ok & np.ones(P[:2] + P[3:], dtype=bool)
        ok[:, :, :, :, 0] = False        # the m loop starts at ms-onx+1
        F = np.zeros(P[:2] + P[3:], order="F")
        F[ok] = np.broadcast_to(flux, F.shape)[ok]
        return "flux", F

    return Experiment("lee_wave_flux", n, d, f0, background, initial, steps, dt=300.0 / fac,
                      fixed=(0.0, 0.0, 0.0), forcing=forcing)


def critical_gm_relax(fac=1.0, steps=3):
    """critical_gm1: nz=160*fac, nm=300*fac, the other axes 1, k_fixed=25.5e-3,
    open z boundaries; the bottom plane relaxes towards a Garrett-Munk
    spectrum E_gm where the z velocity points upward (critical_gm1.f90:11-141)."""
    nz, nm = int(160 * fac), int(300 * fac)
    f0 = f32(1e-4)
    Lz, Ly, Lx = f32(2000.0), 100e3, 100e3
    n = (1, 1, nz, 1, 1, nm)
    d = [np.full(1, Lx / 1), np.full(1, Ly / 1), np.full(nz, Lz / nz),
         np.full(1, f32(0.5e-3)), np.full(1, f32(0.5e-3)), np.full(nm, 2 * PI_F / Lz / 2.0)]
    # (30e-4)**2 is a default-real expression (critical_gm1.f90:64)
    N2 = float(np.float32(30e-4) * np.float32(30e-4))

    def background(m):
        X, Y, Z = _mesh3(m)
        m.Nsqr[:] = N2
        m.U[:] = f32(0.2) * np.exp(-((Z + 1000) * (Z + 1000)) / 200 ** 2)
        m.V[:] = 0.0
        _bottom_fill(m, (m.U,))

    def initial(m, rng):
        m.E[:] = 0.0

    def forcing(m):
        # critical_gm1.f90:85-113 on the bottom plane k = 1
        P, kt, lt, mt, dmt = _forcing_mesh(m)
        g = np.float32(math.gamma(0.5))
        na = float(np.float32(2) * np.float32(1.0) / g / g)   # default-real expression
        nb = 2.0 / PI_F
        E0, jstar = 3e-3, 10
        c1 = 0.0
        dz = m.grid["z"]["dt"]
        for k in range(ONX, ONX + nz):
            c1 = c1 + np.sqrt(m.Nsqr[ONX, ONX, k]) * dz[k] / PI_F
        cstar = c1 / jstar
        N1 = m.Nsqr[:, :, ONX].reshape(P[0], P[1], 1, 1, 1)
        with np.errstate(divide="ignore", invalid="ignore"):
            kh = np.sqrt(kt * kt + lt * lt)
            om = np.sqrt((N1 * (kh * kh) + (f0 * f0) * (mt * mt)) / (kh * kh + mt * mt))
            t = N1 - om * om
            Jac = t * t / ((mt * mt) * om * (N1 - f0 * f0))
            mstar = np.sqrt(N1 - om * om) / cstar
            r = mt / mstar
            funcA = na / (1.0 + r * r)
            funcB = nb * abs(f0) / (om * np.sqrt(om * om - f0 * f0))
            Egm = E0 * funcA / mstar * funcB * Jac
        F = np.asfortranarray(np.broadcast_to(Egm, P[:2] + P[3:]))
        return "relax", F

    return Experiment("critical_gm_relax", n, d, f0, background, initial, steps, dt=30.0,
                      upper=False, lower=False, fixed=(f32(25.5e-3), 0.0, 0.0), forcing=forcing)


# ---------------------------------------------------------------------------
# stretched grids (for_config/gm1.f90, brava.f90): non-uniform spacings
# ---------------------------------------------------------------------------
def gm_column(fac=1, steps=3):
    """gm1: nz=60*fac, nm=80*fac, the other axes 1, k_fixed=50e-3; the m
    spacing is refined towards m=0 and mirrored (gm1.f90:33-49); the initial
    state is a Garrett-Munk spectrum (gm1.f90:52-114)."""
    nz, nm = int(60 * fac), int(80 * fac)
    f0 = f32(1e-4)
    Lz, Ly, Lx = f32(2000.0), 240e3, 240e3
    n = (1, 1, nz, 1, 1, nm)
    dm = grid.symmetric_stretched(nm, -1.0, lo=1e-6, hi=1e-1)
    d = [np.full(1, Lx / 1), np.full(1, Ly / 1), np.full(nz, Lz / nz),
         np.full(1, PI_F / Lx), np.full(1, PI_F / Ly), dm]
    N = 30 * f0                      # N_func, gm1.f90:59

    def background(m):
        X, Y, Z = _mesh3(m)
        m.U[:] = f32(0.10) * (1 + np.tanh((Z + 750) / 150)) / 2.0
        m.Nsqr[:] = N * N
        m.V[:] = 0.0
        _bottom_fill(m, (m.U,))

    def initial(m, rng):
        # gm1.f90:87-114, evaluated on the interior
        sl = _interior(m)
        g = np.float32(math.gamma(0.5))
        na = float(np.float32(2) * np.float32(1.0) / g / g)   # default-real expression
        nb, E0, jstar = 2.0 / PI_F, 3e-3, 15.0
        dz = m.grid["z"]["dt"]
        c1 = 0.0
        for k in range(ONX, ONX + nz):
            c1 = c1 + N * dz[k] / PI_F
        cstar = c1 / jstar
        kt = m.grid["k"]["t"][ONX]
        lt = m.grid["l"]["t"][ONX]
        mt = m.grid["m"]["t"][ONX:ONX + nm]
        kh2 = kt * kt + lt * lt
        om = np.sqrt((N * N * kh2 + (f0 * f0) * (mt * mt)) / (kh2 + mt * mt))
        t = N * N - om * om
        Jac = t * t / ((mt * mt) * om * (N * N - f0 * f0))
        mstar = np.sqrt(N * N - om * om) / cstar
        r = mt / mstar
        funcA = na / (1.0 + r * r)
        funcB = nb * abs(f0) / (om * np.sqrt(om * om - f0 * f0))
        spec = E0 * funcA / mstar * funcB * Jac * N / N / (4 * PI_F)
        m.E[sl] = np.broadcast_to(spec.reshape(1, 1, 1, 1, 1, nm), n)

    return Experiment("gm_column", n, d, f0, background, initial, steps, dt=20.0 / fac,
                      fixed=(f32(50e-3), 0.0, 0.0))


def stretched_mini(n=(8, 6, 8, 6, 6, 8), steps=3, seed=11, upper=True, lower=True, cfl=0.4):
    """The all-axes shear case on non-uniform grids: x spacing growing
    geometrically, y spacing jittered, z refined upward (brava.f90 zgrid),
    k, l, m refined towards zero and mirrored (gm1.f90 / brava.f90 mgrid,
    lgrid)."""
    nx, ny, nz, nk, nl, nm = n
    Lx, Ly, Lz = 30e3, 25e3, 3000.0
    gx = 1.15 ** np.arange(nx)
    jit = 1.0 + 0.3 * np.sin(1.7 * np.arange(ny) + 0.4)
    d = [Lx * gx / gx.sum(), Ly * jit / jit.sum(), grid.bottom_refined(nz, Lz),
         grid.symmetric_stretched(nk, -2e-3), grid.symmetric_stretched(nl, -2e-3),
         grid.symmetric_stretched(nm, -5e-2)]
    base = shear_mini(n=n, steps=steps, seed=seed, upper=upper, lower=lower, cfl=cfl)
    return Experiment("stretched_mini", tuple(n), d, base.f0, base.background, base.initial, steps, cfl=cfl,
                      seed=seed, upper=upper, lower=lower)


# ---------------------------------------------------------------------------
# ensemble member of the batched / served workloads
# ---------------------------------------------------------------------------
SPATIAL_DIMS = (8, 16, 24, 32)
SPECTRAL_DIMS = (8, 12, 16, 24)


def ensemble_member(rng, steps=500, spatial=SPATIAL_DIMS, spectral=SPECTRAL_DIMS, cfl=0.4):
    """One instance: dims per axis drawn from the sets, N0 in [2e-3,1e-2],
    f in [5e-5,1.4e-4], mean-flow amplitude in [0,0.2] m/s, packet init."""
    n = tuple(int(rng.choice(spatial)) for _ in range(3)) + tuple(int(rng.choice(spectral)) for _ in range(3))
    N0 = float(rng.uniform(2e-3, 1e-2))
    f0 = float(rng.uniform(5e-5, 1.4e-4))
    amp = float(rng.uniform(0.0, 0.2))
    seed = int(rng.integers(0, 2 ** 31 - 1))
    nx, ny, nz, nk, nl, nm = n
    # depth 3072 m: Lz/nz is exact in binary for every nz of the sets, so
    # the z grid passes the reference's monotonicity check (calc_grid.f90:261)
    Lx, Ly, Lz = 5e3 * nx, 5e3 * ny, 3072.0
    d = [np.full(nx, Lx / nx), np.full(ny, Ly / ny), np.full(nz, Lz / nz),
         np.full(nk, 4e-3 / nk), np.full(nl, 4e-3 / nl), np.full(nm, 0.1 / nm)]

    def background(m):
        X, Y, Z = _mesh3(m)
        m.Nsqr[:] = (N0 * np.exp(Z / 1000.0)) ** 2
        m.U[:] = amp * np.sin(2 * np.pi * Y / Ly) * np.exp(Z / 500.0)
        m.V[:] = 0.0

    def initial(m, rng2):
        c = (Lx / 2, Ly / 2, -Lz / 2, 1e-3, 0.0, 1e-2)
        _packet(m, rng2, c, 2.0, 1e-3, 1e-8)

    return Experiment("ensemble_member", n, d, f0, background, initial, steps, cfl=cfl, seed=seed,
                      meta={"N0": N0, "f0": f0, "U_amp": amp})
