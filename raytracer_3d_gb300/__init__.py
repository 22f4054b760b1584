"""GB300 (sm_103a) implementation of raytracer_3D's time-stepping path.

The compute lives in libraytracer_gb300.so (CUDA, C ABI in
include/rt_gb300.h); this package is the host-side mirror of the reference
driver's module-state interface (for_src/main_module.f90, main.f90):
`Model.calc_grid`, `Model.calc_parameter`, `Model.integrate`,
`Model.diagnose`.
"""
from .grid import calc_grid, u_centered_grid  # noqa: F401
from .model import Model  # noqa: F401

__all__ = ["Model", "calc_grid", "u_centered_grid"]
