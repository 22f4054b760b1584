"""ctypes wrapper of the CPU oracle (oracle/rt_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs, never by the product path.
Parity status: unpinned by reference outputs (the Fortran reference cannot be
built here and has no tests or golden data); pinned by math known-answer
tests and by committed golden vectors of this oracle.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ONX = 2

FIELDS6 = ("E", "dE", "xdot", "ydot", "zdot", "kdot", "ldot", "mdot", "omega_i", "omega_e",
           "flux_x", "flux_y", "flux_z", "flux_k", "flux_l", "flux_m",
           "lambda_x", "lambda_y", "lambda_z", "meanfl")
FIELDS3 = ("Nsqr", "U", "V", "E_int", "meanfl_int", "diss_ks", "diss_ke", "diss_ls",
           "diss_le", "diss_ms", "diss_me")
AXES = ("x", "y", "z", "k", "l", "m")
FORCING_NONE, FORCING_FLUX, FORCING_RELAX = 0, 1, 2   # ORC_FORCING_* of rt_oracle.h
BUDGET = ("eint", "mflint", "mfl_max", "umax", "vmax", "wmax", "kmax", "lmax", "mmax",
          "bfl_xs", "bfl_xe", "bfl_ys", "bfl_ye", "bfl_zs", "bfl_ze",
          "bfl_ks", "bfl_ke", "bfl_ls", "bfl_le", "bfl_ms", "bfl_me",
          "cfl_x", "cfl_y", "cfl_z", "cfl_k", "cfl_l", "cfl_m", "residual")


class _Budget(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in BUDGET]


_libs = {}


def _load(threads):
    name = "librt_oracle_omp.so" if threads else "librt_oracle.so"
    if name in _libs:
        return _libs[name]
    path = os.path.join(HERE, name)
    if not os.path.exists(path):
        from . import build_oracle  # noqa: F401  (package-relative when imported as oracle.oracle)
        build_oracle.build()
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    lib.orc_create.restype = P
    lib.orc_create.argtypes = [ctypes.c_int] * 6
    lib.orc_destroy.argtypes = [P]
    lib.orc_field.restype = ctypes.POINTER(ctypes.c_double)
    lib.orc_field.argtypes = [P, ctypes.c_int]
    lib.orc_field_len.restype = ctypes.c_longlong
    lib.orc_field_len.argtypes = [P, ctypes.c_int]
    lib.orc_set_scalars.argtypes = [P, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double]
    lib.orc_calc_grid.restype = ctypes.c_int
    lib.orc_calc_grid.argtypes = [P]
    lib.orc_calc_parameter.argtypes = [P]
    lib.orc_integrate.argtypes = [P]
    lib.orc_integrate_n.argtypes = [P, ctypes.c_int]
    lib.orc_diagnose.argtypes = [P, ctypes.POINTER(_Budget)]
    lib.orc_max_rate.restype = ctypes.c_double
    lib.orc_max_rate.argtypes = [P]
    lib.orc_threads.restype = ctypes.c_int
    lib.orc_set_forcing.restype = ctypes.c_int
    lib.orc_set_forcing.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    lib.orc_apply_forcing.argtypes = [P]
    lib.orc_create_light.restype = P
    lib.orc_create_light.argtypes = [ctypes.c_int] * 6
    lib.orc_point_steps.argtypes = [P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int),
                                    ctypes.c_longlong, ctypes.POINTER(ctypes.c_double)]
    _libs[name] = lib
    return lib


class Oracle:
    """Module state of main_module.f90 in C memory, with numpy views."""

    def __init__(self, n, threads=False, light=False):
        """light=True: grids, background and scalars only, for the per-cell
        restatement (point_steps) on fields too large for the arrays"""
        self.n = tuple(int(x) for x in n)
        self.lib = _load(threads)
        self.s = (self.lib.orc_create_light if light else self.lib.orc_create)(*self.n)
        if not self.s:
            raise MemoryError("oracle allocation failed")
        P6 = tuple(x + 2 * ONX for x in self.n)
        P3 = P6[:3]
        for i, name in enumerate(FIELDS6):
            setattr(self, name, None if light else self._view(i, P6))
        for i, name in enumerate(FIELDS3):
            setattr(self, name, self._view(32 + i, P3))
        self.grid = {}
        for a, ax in enumerate(AXES):
            self.grid[ax] = {k: self._view(64 + 4 * a + j, (P6[a],)) for j, k in enumerate(("t", "u", "dt", "du"))}

    def _view(self, fid, shape):
        ptr = self.lib.orc_field(self.s, fid)
        n = int(np.prod(shape))
        assert self.lib.orc_field_len(self.s, fid) == n
        buf = np.ctypeslib.as_array(ptr, shape=(n,))
        return buf.reshape(shape, order="F")

    def close(self):
        if self.s:
            self.lib.orc_destroy(self.s)
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_scalars(self, dt, f0, sign_of_omega_i=1.0, upper=True, lower=True, fixed=(0.0, 0.0, 0.0)):
        self.lib.orc_set_scalars(self.s, dt, f0, sign_of_omega_i, int(upper), int(lower), *fixed)

    def set_spacings(self, d_interior):
        for a, ax in enumerate(AXES):
            self.grid[ax]["dt"][ONX:ONX + self.n[a]] = d_interior[a]

    def calc_grid(self):
        return self.lib.orc_calc_grid(self.s)

    def calc_parameter(self):
        self.lib.orc_calc_parameter(self.s)

    def integrate(self, nsteps=1):
        self.lib.orc_integrate_n(self.s, int(nsteps))

    def set_forcing(self, kind, F=None):
        """set_forcing before every integrate: kind FORCING_NONE, FORCING_FLUX
        (lee1.f90:193-212) or FORCING_RELAX (critical_gm1.f90:119-139); F is
        the padded 5D field (x,y,k,l,m), Fortran order."""
        ptr = None
        if F is not None:
            P5 = tuple(self.n[a] + 2 * ONX for a in (0, 1, 3, 4, 5))
            F = np.asfortranarray(F, dtype=np.float64)
            if F.shape != P5:
                raise ValueError("forcing field must have the padded shape %s, got %s" % (P5, F.shape))
            self._force = F
            ptr = F.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        rc = self.lib.orc_set_forcing(self.s, int(kind), ptr)
        if rc:
            raise ValueError("orc_set_forcing failed (%d)" % rc)

    def apply_forcing(self):
        self.lib.orc_apply_forcing(self.s)

    def diagnose(self):
        b = _Budget()
        self.lib.orc_diagnose(self.s, ctypes.byref(b))
        return {k: getattr(b, k) for k in BUDGET}

    def max_rate(self):
        return self.lib.orc_max_rate(self.s)

    def threads(self):
        return self.lib.orc_threads()

    def point_steps(self, E0, cells):
        """E after one step at the given interior cells (an (K, 6) array of
        Fortran indices i,j,k,l,n,m) from the interior pre-step state E0
        (shape n, any order; copied to Fortran order)"""
        E0 = np.asfortranarray(E0, dtype=np.float64)
        assert E0.shape == self.n
        cells = np.ascontiguousarray(cells, dtype=np.int32)
        assert cells.ndim == 2 and cells.shape[1] == 6
        for a in range(6):
            assert cells[:, a].min() >= 1 and cells[:, a].max() <= self.n[a]
        out = np.empty(len(cells))
        self.lib.orc_point_steps(self.s, E0.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                 cells.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(cells),
                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out
