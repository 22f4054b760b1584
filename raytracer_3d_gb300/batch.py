"""Batched ensemble: many independent wave fields advanced by one
persistent, graph-captured kernel launch per time step (rt_batch_* in
include/rt_gb300.h).

The reference advances one field per run; an ensemble of N fields with
different grids, N(z), f and mean flows is N independent runs of the same
path.  `Batch` keeps each member's `Model` (state, coefficients, dt) and
steps them together.  A member's result is bit-identical to stepping it
alone.
"""
import ctypes

from . import _lib


class Batch:
    def __init__(self, models):
        self.models = list(models)
        self._lib = _lib.load()
        arr = (ctypes.c_void_p * len(self.models))(*[m.handle.value for m in self.models])
        b = ctypes.c_void_p()
        rc = self._lib.rt_batch_create(arr, len(self.models), ctypes.byref(b))
        if rc != 0:
            raise _lib.RtError("rt_batch_create failed (%d): %s" % (rc, self._lib.rt_batch_last_error(None).decode()))
        self._b = b
        for m in self.models:
            m._state_on_device = True
        self.tuning = (8, 256, 0, 16)
        self.persistent = 256
        self.slices = -1
        self.fused = False

    def _check(self, rc, what):
        if rc != 0:
            raise _lib.RtError("%s failed (%d): %s" % (what, rc, self._lib.rt_batch_last_error(self._b).decode()))

    def set_tuning(self, band=8, threads=256, sweep=0, graph_steps=16):
        self._check(self._lib.rt_batch_set_tuning(self._b, band, threads, sweep, graph_steps), "rt_batch_set_tuning")
        self.tuning = (band, threads, sweep, graph_steps)

    def set_persistent(self, threads=256):
        """consumer threads of the warp-specialised class (0: off)"""
        self._check(self._lib.rt_batch_set_persistent(self._b, int(threads)), "rt_batch_set_persistent")
        self.persistent = int(threads)

    def set_slices(self, threads=-1):
        """consumer threads of the small-plane class (0: off, -1: as set_persistent)"""
        self._check(self._lib.rt_batch_set_slices(self._b, int(threads)), "rt_batch_set_slices")
        self.slices = int(threads)

    def set_fused(self, on=True):
        """one launch per step for both warp-specialised classes, or one
        launch per class (the default).  The one-launch form times each
        class's launch when the batch is rebuilt, which waits for the work
        queued before the rebuild."""
        self._check(self._lib.rt_batch_set_fused(self._b, int(bool(on))), "rt_batch_set_fused")
        self.fused = bool(on)

    def persistent_members(self):
        n = self._lib.rt_batch_persistent_members(self._b)
        if n < 0:
            self._check(n, "rt_batch_persistent_members")
        return int(n)

    def integrate(self, nsteps):
        self._check(self._lib.rt_batch_integrate(self._b, int(nsteps)), "rt_batch_integrate")
        for m in self.models:
            m.itt += int(nsteps)

    def sync(self):
        self._check(self._lib.rt_batch_sync(self._b), "rt_batch_sync")

    def stream(self):
        s = ctypes.c_void_p()
        self._check(self._lib.rt_batch_stream(self._b, ctypes.byref(s)), "rt_batch_stream")
        return s.value

    def launch_count(self):
        return int(self._lib.rt_batch_launch_count(self._b))

    @property
    def cells(self):
        return int(self._lib.rt_batch_cells(self._b))

    def close(self):
        if getattr(self, "_b", None):
            self._lib.rt_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
