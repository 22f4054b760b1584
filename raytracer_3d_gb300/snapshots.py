"""NetCDF snapshot files of the reference, written by the host:

  snap3D.cdf  grids, background, and per snapshot the wavenumber integrals
              E_int, meanfl_int, diss_* and the boundary fluxes
              (init_snap3D_cdf, netcdf_io_3D.f90:1-248; diagnose.f90:434-528)
  snap6D.cdf  grids, face velocities, frequencies, and per snapshot E and
              meanfl (init_snap6D_cdf_single, netcdf_io_6D.f90:240-660;
              diagnose.f90:335-380)

Both are NetCDF classic files with 64-bit offsets (CDF-2, NF_64BIT_OFFSET)
and an unlimited Time dimension, written through scipy.io.netcdf_file.  The
schema is the reference's: the same dimension and variable names, Fortran
dimension order reversed into NetCDF's C order (a Fortran (xt,yt,zt,Time)
variable is ('Time','zt','yt','xt')), long_name padded to 24 and units to
16 characters as the reference's character*24 / character*16 attributes
are, and the global attributes f0, k_fixed, l_fixed, m_fixed of
snap3D.cdf.  Variables are defined in the reference's order; scipy's
writer orders them within the file itself (record variables last) and wants
the Time dimension defined first, which readers do not see since they
address dimensions and variables by name.

The data come from the GPU library (rt_get_field, rt_diagnose,
rt_get_state, rt_get_tendency); only omega_i and omega_e, which the library
does not keep, are evaluated here from the dispersion relation
(calc_parameter.f90:13-27), in its operation order.
"""
import os

import numpy as np
from scipy.io import netcdf_file

from .grid import AXES, ONX

TIME_ORIGIN = "01-JAN-1900 00:00:00"
DISS = ("diss_ks", "diss_ke", "diss_ls", "diss_le", "diss_ms", "diss_me")
BFLUX = ("xs", "xe", "ys", "ye", "ks", "ke", "ls", "le", "ms", "me")   # no z (netcdf_io_3D.f90:120-163)
VELOCITIES = ("xdot", "ydot", "zdot", "kdot", "ldot", "mdot")
_VEL_TEXT = ("hor. group velocity", "m/s"), ("hor. group velocity", "m/s"), ("vertical group velocity", "m/s"), \
    ("hor. wavenr. change", "1/ms"), ("hor. wavenr. change", "1/ms"), ("vert. wavenr. change", "1/ms")
_AXIS_TEXT = {"x": ("distance", "m"), "y": ("distance", "m"), "z": ("distance", "m"),
              "k": ("wavenumber", "1/m"), "l": ("wavenumber", "1/m"), "m": ("wavenumber", "1/m")}


def _label(var, long_name, units):
    var.long_name = long_name.ljust(24)[:24]
    var.units = units.ljust(16)[:16]


def _interior1(g, ax, key, n):
    return np.asarray(g[ax][key][ONX:ONX + n], dtype=np.float64)


def _c(a):
    """Fortran-ordered interior array -> NetCDF (C) order"""
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)


def _time_var(f):
    t = f.createVariable("Time", "d", ("Time",))
    _label(t, "Time ", "seconds")
    t.time_origin = TIME_ORIGIN
    return t


def init_snap3d(path, grid, n, Nsqr, U, V, f0, fixed):
    """Create snap3D.cdf (init_snap3D_cdf).  grid: {axis: {"t","u",...}}
    padded; Nsqr/U/V: padded 3D; fixed: (k_fixed, l_fixed, m_fixed)."""
    nx, ny, nz = n[:3]
    with netcdf_file(path, "w", version=2) as f:
        f.createDimension("Time", None)
        for ax, m in (("x", nx), ("y", ny), ("z", nz)):
            f.createDimension(ax + "t", m)
            f.createDimension(ax + "u", m)
        _time_var(f)
        for ax, m in (("x", nx), ("y", ny), ("z", nz)):
            for key in ("t", "u"):
                v = f.createVariable(ax + key, "d", (ax + key,))
                _label(v, "distance", "m")
        sp = ("zt", "yt", "xt")
        for name, text in (("Nsqr", ("buoyancy frequency", "1/s")), ("U", ("mean flow", "m/s")),
                           ("V", ("mean flow", "m/s"))):
            _label(f.createVariable(name, "d", sp), *text)
        for name, text in (("E", ("energy density", "m^2/s^2")), ("meanfl", ("energy change", "m^2/s^3"))):
            _label(f.createVariable(name, "d", ("Time",) + sp), *text)
        for name in DISS:
            _label(f.createVariable(name, "d", ("Time",) + sp), "energy change", "m^2/s^3")
        for b in BFLUX:
            side = "min" if b[1] == "s" else "max"
            _label(f.createVariable("bflux_" + b, "d", ("Time",)), "Energy flux across %s %s" % (side, b[0]), " ")
        _label(f.createVariable("mflint", "d", ("Time",)), "mean flow energy flux", " ")
        f.f0 = float(f0)
        f.k_fixed, f.l_fixed, f.m_fixed = (float(x) for x in fixed)
        sl3 = tuple(slice(ONX, ONX + m) for m in (nx, ny, nz))
        for name, a in (("Nsqr", Nsqr), ("U", U), ("V", V)):
            f.variables[name][:] = _c(np.asarray(a)[sl3])
        for ax, m in (("x", nx), ("y", ny), ("z", nz)):
            for key in ("t", "u"):
                f.variables[ax + key][:] = _interior1(grid, ax, key, m)


def append_snap3d(path, time, fields, budget):
    """Append one snapshot to snap3D.cdf (diagnose.f90:434-528): fields are
    padded 3D arrays E_int, meanfl_int, diss_*; budget the scalar sums."""
    with netcdf_file(path, "a", version=2) as f:
        k = f.variables["Time"].shape[0]
        f.variables["Time"][k] = float(time)
        n = tuple(f.dimensions[d] for d in ("xt", "yt", "zt"))
        sl3 = tuple(slice(ONX, ONX + m) for m in n)
        f.variables["E"][k] = _c(np.asarray(fields["E_int"])[sl3])
        f.variables["meanfl"][k] = _c(np.asarray(fields["meanfl_int"])[sl3])
        for name in DISS:
            f.variables[name][k] = _c(np.asarray(fields[name])[sl3])
        f.variables["mflint"][k] = float(budget["mflint"])
        for b in BFLUX:
            f.variables["bflux_" + b][k] = float(budget["bfl_" + b])
    return k + 1


def dispersion(grid, n, Nsqr, U, V, f0, sign_of_omega_i):
    """omega_i, omega_e on the interior (calc_parameter.f90:13-27), Fortran
    order, in the reference's operation order."""
    sl3 = tuple(slice(ONX, ONX + m) for m in n[:3])
    N3 = np.asarray(Nsqr)[sl3].reshape(n[:3] + (1, 1, 1), order="F")
    U3 = np.asarray(U)[sl3].reshape(n[:3] + (1, 1, 1), order="F")
    V3 = np.asarray(V)[sl3].reshape(n[:3] + (1, 1, 1), order="F")
    kt = _interior1(grid, "k", "t", n[3]).reshape(1, 1, 1, n[3], 1, 1)
    lt = _interior1(grid, "l", "t", n[4]).reshape(1, 1, 1, 1, n[4], 1)
    mt = _interior1(grid, "m", "t", n[5]).reshape(1, 1, 1, 1, 1, n[5])
    kh2 = lt * lt + kt * kt
    mm = mt * mt
    om_i = sign_of_omega_i * np.sqrt((N3 * kh2 + f0 * f0 * mm) / (mm + kh2))
    om_e = om_i + kt * U3 + lt * V3
    return np.asfortranarray(om_i), np.asfortranarray(om_e)


def init_snap6d(path, grid, n, velocities, omega_i, omega_e):
    """Create snap6D.cdf (init_snap6D_cdf_single).  velocities: six padded
    6D arrays (faces 1..n of their own axis are written, as the reference
    writes xdot(1:nx, ...)); omega_i/omega_e: interior 6D arrays."""
    with netcdf_file(path, "w", version=2) as f:
        f.createDimension("Time", None)
        for ax, m in zip(AXES, n):
            f.createDimension(ax + "t", m)
            f.createDimension(ax + "u", m)
        _time_var(f)
        for a, ax in enumerate(AXES):
            text = _AXIS_TEXT[ax]
            _label(f.createVariable(ax + "t", "d", (ax + "t",)), *text)
            _label(f.createVariable(ax + "u", "d", (ax + "u",)), *text)
            _label(f.createVariable("d" + ax + "t", "d", (ax + "u",)), *text)
        t6 = [ax + "t" for ax in AXES]
        for a, name in enumerate(VELOCITIES):
            dims = list(t6)
            dims[a] = AXES[a] + "u"
            _label(f.createVariable(name, "d", tuple(reversed(dims))), *_VEL_TEXT[a])
        c6 = tuple(reversed(t6))
        _label(f.createVariable("omega_i", "d", c6), "intrinsic frequency", "1/s")
        _label(f.createVariable("omega_e", "d", c6), "extrinsic frequency", "1/s")
        _label(f.createVariable("E", "d", ("Time",) + c6), "energy density", "m^5/s^2")
        _label(f.createVariable("meanfl", "d", ("Time",) + c6), "energy change", "m^5/s^3")
        for a, ax in enumerate(AXES):
            f.variables[ax + "t"][:] = _interior1(grid, ax, "t", n[a])
            f.variables[ax + "u"][:] = _interior1(grid, ax, "u", n[a])
            f.variables["d" + ax + "t"][:] = _interior1(grid, ax, "dt", n[a])
        sl6 = tuple(slice(ONX, ONX + m) for m in n)
        for name, v in zip(VELOCITIES, velocities):
            f.variables[name][:] = _c(np.asarray(v)[sl6])
        f.variables["omega_i"][:] = _c(omega_i)
        f.variables["omega_e"][:] = _c(omega_e)


def append_snap6d(path, time, E, meanfl):
    """Append E and meanfl (interior 6D, Fortran order) as one snapshot
    (diagnose.f90:335-380)."""
    with netcdf_file(path, "a", version=2) as f:
        k = f.variables["Time"].shape[0]
        f.variables["Time"][k] = float(time)
        f.variables["E"][k] = _c(E)
        f.variables["meanfl"][k] = _c(meanfl)
    return k + 1


class Snapshots:
    """init_diag / the output part of diagnose for a Model: create the files
    once the coefficients are known, then write() one snapshot after a
    step (main.f90:61, :74)."""

    def __init__(self, model, directory=".", write_6d=True):
        self.model = model
        self.write_6d = bool(write_6d)
        self.path3d = os.path.join(directory, "snap3D.cdf")
        self.path6d = os.path.join(directory, "snap6D.cdf")
        m = model
        init_snap3d(self.path3d, m.grid, m.n, m.Nsqr, m.U, m.V, m.f0, m.fixed)
        if self.write_6d:
            vel = [m.get_field(a) for a in range(6)]
            om_i, om_e = dispersion(m.grid, m.n, m.Nsqr, m.U, m.V, m.f0, m.sign_of_omega_i)
            init_snap6d(self.path6d, m.grid, m.n, vel, om_i, om_e)

    def write(self):
        """One snapshot at time itt*dt of the last step; returns the budget."""
        m = self.model
        budget, fields = m.diagnose(fields=True)
        t = m.itt * m.dt
        append_snap3d(self.path3d, t, fields, budget)
        if self.write_6d:
            sl = tuple(slice(ONX, ONX + k) for k in m.n)
            E = m.get_state()
            E = np.asarray(E[sl] if getattr(m, "padded", True) else E, dtype=np.float64)
            _, meanfl = m.get_tendency()
            append_snap6d(self.path6d, t, E, meanfl[sl])
        return budget
