"""CPU checks of the stretched grids (for_config/gm1.f90:33-49,
brava.f90:32-58): the bisection, the closure conditions, the monotonicity
that calc_grid.f90:260-293 demands, and that the host grid construction and
the oracle's calc_grid agree bit for bit on non-uniform spacings."""
import numpy as np
import pytest

from harness import ONX, build_oracle, configs, interior
from raytracer_3d_gb300 import grid

F32 = np.float32


def test_bisection_finds_a_binary32_root():
    r = grid.bisect(lambda x: F32(F32(x * x) - F32(2)), 0.0, 2.0, 1e-7)
    assert abs(float(r) - 2 ** 0.5) < 2e-7
    assert F32(r * r) - F32(2) <= 0
    # a decreasing function: the end with f <= 0 is the upper one
    r = grid.bisect(lambda x: F32(F32(1) - x), 0.0, 4.0, 1e-7)
    assert abs(float(r) - 1.0) < 2e-7


def test_bisection_rejects_an_unbracketed_interval():
    with pytest.raises(grid.GridError):
        grid.bisect(lambda x: F32(x * x + F32(1)), -1.0, 1.0, 1e-6)


def test_bisection_terminates_below_the_binary32_spacing():
    # width 990 needs 37 halvings to fall below 1e-8, far below the binary32
    # spacing near the root; the nominal width still shrinks
    r = grid.bisect(lambda x: F32(x - F32(123.456)), 10.0, 1000.0, 1e-8)
    assert abs(float(r) - 123.456) < 1e-4


@pytest.mark.parametrize("n,start", [(80, -1.0), (320, -1.0), (6, -2e-3), (8, -5e-2), (20, -0.02)])
def test_symmetric_stretched_axis(n, start):
    d = grid.symmetric_stretched(n, start, lo=1e-6 if start == -1.0 else None,
                                 hi=1e-1 if start == -1.0 else None)
    half = n // 2
    assert d.shape == (n,) and (d > 0).all()
    assert np.array_equal(d[:half], d[half:][::-1])                  # mirrored about zero
    assert (np.diff(d[:half]) <= 0).all()                            # refined towards zero
    # closure: start + sum of the first half + the last spacing again = 0
    p = F32(start)
    for v in d[:half]:
        p = F32(p + F32(v))
    # to the binary32 rounding of the half-axis sum
    assert abs(float(F32(p + F32(d[half - 1])))) <= half * np.spacing(F32(abs(start)))
    assert d[half - 1] / d[0] == pytest.approx(0.2, rel=1e-5)        # 1 - 0.8 at the centre


@pytest.mark.parametrize("nz,Lz", [(20, 2000.0), (8, 3000.0), (60, 4000.0)])
def test_bottom_refined_axis(nz, Lz):
    d = grid.bottom_refined(nz, Lz)
    assert d.shape == (nz,) and (d > 0).all()
    assert (np.diff(d) <= 0).all()                                   # calc_grid.f90:260-270
    # z(0) = -Lz - d(1)/2 and the last centre lies at z = 0: z(nz) = -d(nz)/2
    assert float(d.sum()) == pytest.approx(Lz + d[0] / 2 - d[-1] / 2, rel=1e-5)


def test_small_axes_are_refused():
    with pytest.raises(grid.GridError):
        grid.symmetric_stretched(2, -1.0)
    with pytest.raises(grid.GridError):
        grid.symmetric_stretched(7, -1.0)


@pytest.mark.parametrize("make", [lambda: configs.gm_column(), lambda: configs.stretched_mini(),
                                  lambda: configs.stretched_mini(n=(4, 4, 4, 4, 4, 4))])
def test_host_grid_equals_oracle_grid(make):
    exp = make()
    o = build_oracle(exp)
    g = grid.calc_grid(exp.n, exp.d_interior, exp.fixed)
    for ax in grid.AXES:
        for k in ("t", "u", "dt", "du"):
            assert np.array_equal(g[ax][k], o.grid[ax][k]), (ax, k)
    # spectral centres are symmetric about zero on the mirrored axes
    for a, ax in ((3, "k"), (4, "l"), (5, "m")):
        if exp.n[a] > 1:
            t = g[ax]["t"][ONX:ONX + exp.n[a]]
            assert np.allclose(t, -t[::-1], rtol=0, atol=1e-12 * np.abs(t).max())


def test_stretched_cases_are_stable_and_close_the_budget():
    for exp in (configs.gm_column(), configs.stretched_mini()):
        o = build_oracle(exp)
        sl = interior(exp.n)
        assert np.isfinite(o.E[sl]).all() and o.E[sl].max() > 0
        o.integrate(4)
        b = o.diagnose()
        assert np.isfinite(o.E[sl]).all()
        scale = abs(b["eint"]) + abs(b["mflint"]) + 1e-300
        assert abs(b["residual"]) <= 1e-10 * scale
