"""Generate the golden fixtures of the path from the CPU oracle.

The reference ships no golden data and cannot be built here, so these
fixtures pin the oracle (and through it the GPU library) against
regressions: for each case the final interior state, the budget of the last
step, the 3D wavenumber integrals and a SHA-256 of the interior after every
step.  Inputs are the seeded experiments of raytracer_3d_gb300.configs.

    python tests/golden/make_golden.py [case ...]     # all cases by default
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from harness import ONX, build_oracle, interior  # noqa: E402
from raytracer_3d_gb300 import configs  # noqa: E402

CASES = {
    "shear_mini": (lambda: configs.shear_mini(), 5),
    "shear_open_neg": (lambda: configs.shear_mini(n=(5, 6, 4, 4, 6, 4), upper=False, lower=False,
                                                  sign_of_omega_i=-1.0, seed=3), 5),
    "column_1d": (lambda: configs.column_1d(fac=1), 8),
    "section_2d": (lambda: configs.section_2d(fac=0.5), 4),
    # bottom forcing (lee1.f90:193-229, critical_gm1.f90:119-141)
    "lee_wave_flux": (lambda: configs.lee_wave_flux(fac=1, nz=10), 8),
    "critical_gm_relax": (lambda: configs.critical_gm_relax(fac=0.2), 8),
    # non-uniform spacings on every axis (gm1.f90 / brava.f90 grid forms)
    "stretched_mini": (lambda: configs.stretched_mini(n=(6, 4, 6, 4, 4, 4)), 5),
}

DIAG3 = ("E_int", "meanfl_int", "diss_ks", "diss_ke", "diss_ls", "diss_le", "diss_ms", "diss_me")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_case(name):
    make, steps = CASES[name]
    exp = make()
    o = build_oracle(exp)
    sl = interior(exp.n)
    # inputs, stored so that the fixtures do not depend on the platform's
    # transcendental functions that generated them
    inputs = {"in_Nsqr": o.Nsqr.copy(), "in_U": o.U.copy(), "in_V": o.V.copy(), "in_E": o.E.copy()}
    for a, ax in enumerate("xyzklm"):
        inputs["in_d" + ax] = np.asarray(exp.d_interior[a], dtype=np.float64)
    kind = None
    if exp.forcing is not None:   # the interior of the forcing field (its ghosts are never read)
        kind, F = exp.forcing(o)
        inputs["in_F"] = F[tuple(slice(ONX, ONX + exp.n[a]) for a in (0, 1, 3, 4, 5))].copy()
    hashes = []
    for _ in range(steps):
        o.integrate(1)
        hashes.append(digest(o.E[sl]))
    budget = o.diagnose()
    sl3 = interior(exp.n[:3])
    arrays = dict(inputs)
    arrays["E"] = o.E[sl].copy()
    for k in DIAG3:
        arrays[k] = getattr(o, k)[sl3].copy()
    meta = {"case": name, "n": list(exp.n), "steps": steps, "dt": o.dt, "step_sha256": hashes,
            "budget": budget, "f0": exp.f0, "sign_of_omega_i": exp.sign_of_omega_i, "upper": exp.upper,
            "lower": exp.lower, "fixed": list(exp.fixed), "cfl": exp.cfl, "forcing": kind}
    return meta, arrays


def main(names=None):
    for name in names or CASES:
        meta, arrays = run_case(name)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(meta, f, indent=1, sort_keys=True)
        print(name, meta["n"], meta["steps"], "steps")


if __name__ == "__main__":
    main(sys.argv[1:])
