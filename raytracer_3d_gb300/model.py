"""Host-side mirror of the reference driver's module-state interface.

The reference keeps its model in module variables (for_src/main_module.f90:
41-77) and steps it with argument-free subroutines called from the main
loop (for_src/main.f90:36-79):

    set_parameter; allocate_main_module; set_grid; calc_grid;
    set_initial_conditions; calc_parameter
    do: set_forcing; integrate; diagnose (every snapint/dt steps)

`Model` holds the same host arrays (padded, Fortran order) and exposes the
same steps, with calc_parameter / integrate / the diagnose budget executed
by libraytracer_gb300.so on the GPU.  Host arrays are numpy float64 in
Fortran order so that a 6D array indexes as E[i, j, k, l, n, m] with Fortran
index f at position f + 1.
"""
import ctypes

import numpy as np

from . import _lib
from .grid import AXES, ONX, calc_grid

PRECISIONS = {"fp64": _lib.RT_FP64, "fp32": _lib.RT_FP32}


def padded_shape(n):
    return tuple(int(x) + 2 * ONX for x in n)


def zeros_padded(n):
    return np.zeros(padded_shape(n), dtype=np.float64, order="F")


class Model:
    """One wave field on one GPU: the module state of main_module.f90 plus a
    device handle of libraytracer_gb300.so."""

    def __init__(self, nx, ny, nz, nk, nl, nm, *, dt, f0=1e-4, sign_of_omega_i=1.0,
                 enable_upper_reflection=True, enable_lower_reflection=True,
                 precision="fp64", k_fixed=0.0, l_fixed=0.0, m_fixed=0.0, padded=True):
        self.n = (nx, ny, nz, nk, nl, nm)
        self.dt = float(dt)
        self.f0 = float(f0)
        self.sign_of_omega_i = float(sign_of_omega_i)
        self.enable_upper_reflection = bool(enable_upper_reflection)
        self.enable_lower_reflection = bool(enable_lower_reflection)
        self.precision = precision
        self.fixed = (float(k_fixed), float(l_fixed), float(m_fixed))
        self.itt = 0
        # host arrays of allocate_main_module (main_module.f90:131-232); with
        # padded=False the host state is the interior only (no ghost cells),
        # moved by rt_set_state_interior / rt_get_state_interior
        self.padded = bool(padded)
        self.E = zeros_padded(self.n) if self.padded else np.zeros(self.n, order="F")
        n3 = self.n[:3]
        self.Nsqr = zeros_padded(n3)
        self.U = zeros_padded(n3)
        self.V = zeros_padded(n3)
        self.grid = None
        self._lib = _lib.load()
        dims = _lib.RtDims(nx, ny, nz, nk, nl, nm, ONX)
        par = _lib.RtParams(self.dt, self.f0, self.sign_of_omega_i,
                            int(self.enable_upper_reflection), int(self.enable_lower_reflection),
                            PRECISIONS[precision])
        h = ctypes.c_void_p()
        rc = self._lib.rt_create(ctypes.byref(dims), ctypes.byref(par), ctypes.byref(h))
        _lib.check(rc, None, "rt_create")
        self._h = h
        self._state_on_device = False

    # ---- lifetime -----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.rt_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc, what):
        return _lib.check(rc, self._h, what)

    # ---- setup (main.f90:36-47) ----------------------------------------------
    def calc_grid(self, d_interior):
        """set_grid + calc_grid: interior spacings -> padded grids."""
        self.grid = calc_grid(self.n, d_interior, self.fixed)
        for ax in AXES:  # xt, xu, dxt, dxu, ... as in main_module.f90:66-77
            g = self.grid[ax]
            setattr(self, ax + "t", g["t"])
            setattr(self, ax + "u", g["u"])
            setattr(self, "d" + ax + "t", g["dt"])
            setattr(self, "d" + ax + "u", g["du"])
        return self.grid

    def coord(self, ax, key="t"):
        return self.grid[ax][key]

    def calc_parameter(self):
        """calc_parameter (calc_parameter.f90:2-264) on the GPU."""
        g = self.grid
        arrs = [np.ascontiguousarray(g[ax]["dt"]) for ax in AXES]
        arrs += [np.ascontiguousarray(g[ax]["t"]) for ax in ("k", "l", "m")]
        self._check(self._lib.rt_set_grid(self._h, *[_lib.dptr(a) for a in arrs]), "rt_set_grid")
        self._check(self._lib.rt_set_background(self._h, _lib.dptr(self.Nsqr), _lib.dptr(self.U),
                                                _lib.dptr(self.V)), "rt_set_background")
        self._check(self._lib.rt_calc_parameter(self._h), "rt_calc_parameter")

    def max_rate(self):
        r = ctypes.c_double()
        self._check(self._lib.rt_max_rate(self._h, ctypes.byref(r)), "rt_max_rate")
        return r.value

    def set_dt(self, dt):
        self.dt = float(dt)
        self._check(self._lib.rt_set_dt(self._h, self.dt), "rt_set_dt")

    def get_field(self, which):
        out = zeros_padded(self.n)
        self._check(self._lib.rt_get_field(self._h, which, _lib.dptr(out)), "rt_get_field")
        return out

    # ---- state ----------------------------------------------------------------
    def set_state(self):
        """Upload the host E (interior) to the device."""
        if self.padded:
            self._check(self._lib.rt_set_state(self._h, _lib.dptr(self.E)), "rt_set_state")
        else:
            dt = np.float64 if self.precision == "fp64" else np.float32
            src = np.asfortranarray(self.E, dtype=dt)
            self._check(self._lib.rt_set_state_interior(self._h, src.ctypes.data_as(ctypes.c_void_p)),
                        "rt_set_state_interior")
        self._state_on_device = True

    def set_host_access(self, direct=True):
        """direct: the GPU reads / writes the host array in place when the
        device supports pageable memory access; else pinned staging."""
        self._check(self._lib.rt_set_host_access(self._h, 1 if direct else 0), "rt_set_host_access")

    def host_direct(self):
        return bool(self._lib.rt_host_direct(self._h))

    def get_state(self):
        """Download the device E into the host array (interior).  With
        padded=False it returns a new interior array in the handle's
        precision (binary32 for the fp32 form)."""
        if not self.padded:
            out = np.empty(self.n, dtype=np.float64 if self.precision == "fp64" else np.float32, order="F")
            self._check(self._lib.rt_get_state_interior(self._h, out.ctypes.data_as(ctypes.c_void_p)),
                        "rt_get_state_interior")
            return out
        self._check(self._lib.rt_get_state(self._h, _lib.dptr(self.E)), "rt_get_state")
        return self.E

    def get_tendency(self):
        """dE (after the mean-flow term) and meanfl of the last step, as
        padded 6D arrays (rt_get_tendency); zeros before the first step, as
        the reference allocates them."""
        dE, mfl = zeros_padded(self.n), zeros_padded(self.n)
        rc = self._lib.rt_get_tendency(self._h, _lib.dptr(dE), _lib.dptr(mfl))
        if rc == _lib.RT_ERR_STATE and self.itt == 0:
            return dE, mfl
        self._check(rc, "rt_get_tendency")
        return dE, mfl

    # ---- phase timers (timing_module.f90 tic / toc) -----------------------------
    def tic(self, name):
        """start the named phase timer (a CUDA event on the handle's stream)"""
        self._check(self._lib.rt_tic(self._h, name.encode()), "rt_tic")

    def toc(self, name):
        self._check(self._lib.rt_toc(self._h, name.encode()), "rt_toc")

    def timing_secs(self, name):
        """(device seconds, tic/toc pairs) accumulated for the named phase"""
        secs, calls = ctypes.c_double(), ctypes.c_longlong()
        self._check(self._lib.rt_timing_secs(self._h, name.encode(), ctypes.byref(secs), ctypes.byref(calls)),
                    "rt_timing_secs")
        return secs.value, calls.value

    def timed(self, name):
        """context manager: tic on entry, toc on exit"""
        model = self

        class _Phase:
            def __enter__(self):
                model.tic(name)
                return model

            def __exit__(self, *exc):
                model.toc(name)
                return False
        return _Phase()

    def timing_summary(self, names=("main loop", "integrate", "diag")):
        """the reference's end-of-run summary (main.f90:86-101) for the
        named phases, as text"""
        lines = []
        for n in names:
            secs, calls = self.timing_secs(n)
            lines.append("%-25s = %12.4f s  (%d calls)" % (n, secs, calls))
        return "\n".join(lines)

    # ---- bottom forcing (set_forcing, main.f90:69) ------------------------------
    FORCING = {"none": _lib.RT_FORCING_NONE, "flux": _lib.RT_FORCING_FLUX, "relax": _lib.RT_FORCING_RELAX}

    def forcing_shape(self):
        """Padded shape of a forcing field: axes x,y,k,l,m."""
        return tuple(self.n[a] + 2 * ONX for a in (0, 1, 3, 4, 5))

    def set_forcing(self, kind, F=None):
        """Apply a bottom forcing before every following step: kind "flux"
        (E += dt*F/dzt(1), lee1.f90:193-212), "relax" (E -= dt*max(0,zdot)*
        (E-F)/dzt(1), critical_gm1.f90:119-139) or "none".  F is the padded
        5D field with axes x,y,k,l,m (forcing_shape()), Fortran order."""
        code = self.FORCING[kind] if isinstance(kind, str) else int(kind)
        ptr = None
        if code != _lib.RT_FORCING_NONE:
            F = np.asfortranarray(F, dtype=np.float64)
            if F.shape != self.forcing_shape():
                raise ValueError("forcing field must have the padded shape %s, got %s"
                                 % (self.forcing_shape(), F.shape))
            ptr = _lib.dptr(F)
        self._check(self._lib.rt_set_forcing(self._h, code, ptr), "rt_set_forcing")

    # ---- time stepping (main.f90:64-79) ----------------------------------------
    def integrate(self, nsteps=1):
        """integrate (integrate.f90:4-271), nsteps times, state on the GPU."""
        if not self._state_on_device:
            self.set_state()
        self._check(self._lib.rt_integrate(self._h, int(nsteps)), "rt_integrate")
        self.itt += int(nsteps)

    def integrate_host(self):
        """One integrate on the host array (upload, step, download)."""
        if not self.padded:
            raise ValueError("integrate_host needs the padded host array (Model(..., padded=True))")
        self._check(self._lib.rt_integrate_host(self._h, _lib.dptr(self.E)), "rt_integrate_host")
        self._state_on_device = True
        self.itt += 1

    def diagnose(self, fields=True):
        """Budget part of diagnose (diagnose.f90:46-329) for the last step.
        Returns (budget dict, dict of padded 3D arrays or None)."""
        b = _lib.RtBudget()
        names = ("E_int", "meanfl_int", "diss_ks", "diss_ke", "diss_ls", "diss_le", "diss_ms", "diss_me")
        arrs = {k: zeros_padded(self.n[:3]) for k in names} if fields else None
        ptrs = [_lib.dptr(arrs[k]) if fields else None for k in names]
        self._check(self._lib.rt_diagnose(self._h, ctypes.byref(b), *ptrs), "rt_diagnose")
        return {k: getattr(b, k) for k in _lib.BUDGET_FIELDS}, arrs

    # ---- plumbing ---------------------------------------------------------------
    # rt_set_tuning codes (4-8, 10-12 and 17 belonged to removed binary32 kernels)
    VARIANTS = {"plane": 0, "cell": 1, "tma": 2, "group": 3, "w3": 9, "w6": 13, "w2z": 14, "split": 15, "fast": 16, "w2q": 18}

    def set_tuning(self, variant="tma", band=8, threads=512, sweep=0):
        """Schedule of the step kernel; never changes results."""
        self._check(self._lib.rt_set_tuning(self._h, self.VARIANTS[variant], int(band), int(threads)),
                    "rt_set_tuning")
        self._check(self._lib.rt_set_schedule_sweep(self._h, int(sweep)), "rt_set_schedule_sweep")

    def sync(self):
        self._check(self._lib.rt_sync(self._h), "rt_sync")

    @property
    def handle(self):
        return self._h

    def stream(self):
        s = ctypes.c_void_p()
        self._check(self._lib.rt_stream(self._h, ctypes.byref(s)), "rt_stream")
        return s.value

    def launch_count(self):
        return int(self._lib.rt_launch_count(self._h))

    def device_bytes(self):
        return int(self._lib.rt_device_bytes(self._h))
