"""Load the committed golden fixtures (tests/golden/) as experiments whose
inputs come from the fixture files, not from regenerating them."""
import json
import os

import numpy as np

from raytracer_3d_gb300.configs import Experiment

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ("shear_mini", "shear_open_neg", "column_1d", "section_2d", "lee_wave_flux", "critical_gm_relax",
         "stretched_mini")
# cases the GPU test checks against the fixtures directly; the forced and
# stretched ones reach the GPU through the oracle (bit-identical parity tests)
GPU_NAMES = NAMES[:4]


def load(name):
    with open(os.path.join(HERE, name + ".json")) as f:
        meta = json.load(f)
    arrs = dict(np.load(os.path.join(HERE, name + ".npz")))
    n = tuple(meta["n"])

    def background(m):
        m.Nsqr[:] = arrs["in_Nsqr"]
        m.U[:] = arrs["in_U"]
        m.V[:] = arrs["in_V"]

    def initial(m, rng):
        m.E[:] = arrs["in_E"]

    forcing = None
    if meta.get("forcing"):
        def forcing(m):
            F = np.zeros(tuple(n[a] + 4 for a in (0, 1, 3, 4, 5)), order="F")
            F[tuple(slice(2, 2 + n[a]) for a in (0, 1, 3, 4, 5))] = arrs["in_F"]
            return meta["forcing"], F

    d = [arrs["in_d" + ax] for ax in "xyzklm"]
    exp = Experiment(name, n, d, meta["f0"], background, initial, meta["steps"],
                     dt=None if meta["cfl"] else meta["dt"], cfl=meta["cfl"],
                     sign_of_omega_i=meta["sign_of_omega_i"], upper=meta["upper"], lower=meta["lower"],
                     fixed=tuple(meta["fixed"]), forcing=forcing)
    return exp, meta, arrs
