"""The per-cell restatement of the oracle (orc_point_steps, for spot checks
of fields too large for the whole-array oracle) against the whole-array
oracle: the state after one step, at every interior cell of the small
cases (all-axes shear flow with reflection on, off and mixed, the negative
frequency branch, ragged and minimum sizes, the reference's 1D and 2D
setups with the analytic velocity branch, stretched grids), must be
bit-identical, and it must stay so after a few steps have built gradients
at the boundaries."""
import numpy as np
import pytest

from harness import build_oracle, build_point_oracle, configs, interior

CASES = {
    "shear_mini": lambda: configs.shear_mini(),
    "shear_open": lambda: configs.shear_mini(upper=False, lower=False),
    "shear_mixed_neg": lambda: configs.shear_mini(upper=True, lower=False, sign_of_omega_i=-1.0),
    "ragged": lambda: configs.shear_mini(n=(7, 3, 5, 2, 6, 4)),
    "min_n2": lambda: configs.shear_mini(n=(2, 2, 2, 2, 2, 2)),
    "column_1d": lambda: configs.column_1d(fac=1),
    "section_2d": lambda: configs.section_2d(fac=0.5),
    "stretched": lambda: configs.stretched_mini(),
    "stretched_open": lambda: configs.stretched_mini(n=(8, 8, 6, 4, 6, 4), upper=False, lower=False),
    "jet_small": lambda: configs.jet_large(n=(8, 8, 8, 8, 8, 8)),
}


@pytest.mark.parametrize("name", list(CASES))
def test_point_steps_equal_the_whole_array_oracle(name):
    exp = CASES[name]()
    o = build_oracle(exp)
    po = build_point_oracle(exp, o.dt, threads=False)
    sl = interior(exp.n)
    cells = np.stack(np.meshgrid(*[np.arange(1, k + 1) for k in exp.n], indexing="ij"), axis=-1)
    cells = cells.reshape(-1, 6).astype(np.int32)
    try:
        for s in range(3):
            E0 = o.E[sl].copy(order="F")
            o.integrate(1)
            got = po.point_steps(E0, cells)
            ref = np.array([o.E[tuple(int(c) + 1 for c in cell)] for cell in cells])
            assert np.array_equal(got, ref), (name, s, float(np.max(np.abs(got - ref))))
    finally:
        po.close()
        o.close()
