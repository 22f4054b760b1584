"""Parity of the GPU path (through the C ABI) with the CPU oracle.

The plain binary64 form reproduces the reference's arithmetic operation by
operation, so coefficients, every state after every step and the
wavenumber-integrated budget fields must be bit-identical; the scalar budget
sums are reduced in a different order and must agree to 1e-12 relative.
(The required tolerance for the FP64 form is 1e-12 relative L-infinity per
step; the tests assert the stronger bit-identity and report it.)
"""
import ctypes

import numpy as np
import pytest

from harness import ONX, build_oracle, configs, face_range, interior, max_rel, rounding_noise_bound

pytestmark = pytest.mark.gpu

FP64_STEP_TOL = 1e-12   # relative L-inf per step (the stated bound)


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()


CASES = {
    "shear_mini": lambda: configs.shear_mini(),
    "shear_open": lambda: configs.shear_mini(upper=False, lower=False),
    "shear_mixed_neg": lambda: configs.shear_mini(upper=True, lower=False, sign_of_omega_i=-1.0),
    "ragged": lambda: configs.shear_mini(n=(7, 3, 5, 2, 6, 4)),
    "min_n2": lambda: configs.shear_mini(n=(2, 2, 2, 2, 2, 2)),
    "column_1d": lambda: configs.column_1d(fac=1),
    "section_2d": lambda: configs.section_2d(fac=0.5),
    "packet_small": lambda: configs.packet_small(),
    "stretched": lambda: configs.stretched_mini(),
    "stretched_open": lambda: configs.stretched_mini(n=(8, 8, 6, 4, 6, 4), upper=False, lower=False),
    "gm_column": lambda: configs.gm_column(),
}

VEL = ("xdot", "ydot", "zdot", "kdot", "ldot", "mdot")


def _pair(name, precision="fp64"):
    exp = CASES[name]()
    m = configs.build_model(exp, precision)
    o = build_oracle(exp)
    return exp, m, o


@pytest.mark.parametrize("name", list(CASES))
def test_coefficients_bit_identical(name):
    exp, m, o = _pair(name)
    from raytracer_3d_gb300 import _lib
    try:
        assert m.max_rate() == o.max_rate()
        assert m.dt == o.dt
        for a, v in enumerate(VEL):
            got = m.get_field(a)
            sl = face_range(exp.n, a)
            ref = getattr(o, v)[sl]
            assert np.array_equal(got[sl], ref), (v, max_rel(got[sl], ref))
        sl = interior(exp.n)
        for c, lam in enumerate(("lambda_x", "lambda_y", "lambda_z")):
            got = m.get_field(_lib.RT_F_LAMBDA_X + c)
            assert np.array_equal(got[sl], getattr(o, lam)[sl]), lam
    finally:
        m.close()


SCHEDULES = [("tma", 8, 1024, 0), ("tma", 3, 128, 1), ("tma", 1, 512, 0), ("plane", 8, 256, 0),
             ("plane", 2, 512, 1), ("group", 8, 256, 0), ("group", 3, 1024, 1), ("group", 2, 128, 0),
             ("w3", 8, 256, 0), ("w3", 3, 512, 1), ("w3", 4, 128, 0), ("w6", 8, 256, 0), ("w6", 3, 512, 1),
             ("w2z", 8, 512, 1), ("w2z", 3, 256, 0), ("w2z", 4, 128, 0), ("w2q", 8, 512, 1), ("w2q", 3, 256, 0),
             ("cell", 8, 256, 0), ("split", 8, 256, 0)]


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("sched", SCHEDULES, ids=lambda s: "%s-b%d-t%d-s%d" % s)
def test_steps_bit_identical(name, sched):
    exp, m, o = _pair(name)
    m.set_tuning(*sched)
    sl = interior(exp.n)
    try:
        nsteps = 2 if name == "packet_small" else 4
        for s in range(nsteps):
            m.integrate(1)
            o.integrate(1)
            m.get_state()
            rel = max_rel(m.E[sl], o.E[sl])
            assert rel <= FP64_STEP_TOL, (s, rel)
            assert np.array_equal(m.E[sl], o.E[sl]), (s, rel)
    finally:
        m.close()


@pytest.mark.parametrize("name", list(CASES))
def test_fast_fp64_within_bound(name):
    """the fast binary64 schedule (no divisions, integer-selected limiter,
    regrouped update) stays within the plain form's bound of 1e-12 relative
    L-infinity of the oracle at every step"""
    exp, m, o = _pair(name)
    m.set_tuning("fast", 8, 256)
    sl = interior(exp.n)
    worst = 0.0
    try:
        for s in range(4):
            m.integrate(1)
            o.integrate(1)
            m.get_state()
            rel = max_rel(m.E[sl], o.E[sl])
            worst = max(worst, rel)
            assert rel <= FP64_STEP_TOL, (s, rel)
        print("%s: fast binary64 within %.2e of the oracle over 4 steps" % (name, worst))
    finally:
        m.close()


@pytest.mark.parametrize("n", [(7, 3, 5, 2, 6, 10), (8, 8, 8, 4, 2, 6), (33, 2, 4, 2, 4, 8)])
def test_fast_fp64_band_order_invariant(n):
    """the band only orders the spectral planes among the CTAs (a width that
    does not divide nm is reduced to one that does): every band gives the
    same bits"""
    exp = configs.shear_mini(n=n)
    outs = []
    for band in (1, 2, 3, 4, 8, 64):
        m = configs.build_model(exp, "fp64")
        m.set_tuning("fast", band, 256)
        m.integrate(3)
        outs.append(m.get_state()[interior(exp.n)].copy())
        m.close()
    for b, out in zip((2, 3, 4, 8, 64), outs[1:]):
        assert np.array_equal(out, outs[0]), b


def test_fast_fp64_switches_with_bit_exact_schedules():
    """switching between the fast and the bit-exact schedules on one handle
    (the per-face cache changes meaning between uCFL and h) keeps every
    step on its own bound: each step starts from the oracle's state"""
    exp, m, o = _pair("shear_mini")
    sl = interior(exp.n)
    try:
        for sched in ("fast", "tma", "fast", "split", "plane", "fast", "group"):
            m.E[sl] = o.E[sl]
            m.set_state()
            m.set_tuning(sched, 8, 256)
            m.integrate(1)
            o.integrate(1)
            m.get_state()
            if sched == "fast":
                assert max_rel(m.E[sl], o.E[sl]) <= FP64_STEP_TOL, sched
            else:
                assert np.array_equal(m.E[sl], o.E[sl]), sched
    finally:
        m.close()


def vol_widths(o, n):
    return [o.grid["xyzklm"[a]]["dt"][ONX:ONX + n[a]] for a in range(6)]


def _vol(o, n):
    vol = np.ones(n)
    for a in range(6):
        shp = [1] * 6
        shp[a] = n[a]
        vol = vol * o.grid["xyzklm"[a]]["dt"][ONX:ONX + n[a]].reshape(shp)
    return vol


def test_packet_8x8x16x16e3_200_steps():
    """the 8x8x16 x 16^3 packet workload run to its full 200 steps: the
    two-pass bit-exact schedule equals the oracle bit for bit at every
    snapshot step, the fast schedule stays within 1e-12 relative L-infinity,
    and after the last step the budget (diagnose.f90:46-329) matches the
    oracle's, with a residual at round-off and the total energy sum(E*vol)
    equal"""
    exp = CASES["packet_small"]()
    o = build_oracle(exp, threads=True)
    exact = configs.build_model(exp, "fp64")
    fast = configs.build_model(exp, "fp64")
    exact.set_tuning("split", 8, 256)
    fast.set_tuning("fast", 8, 256)
    sl = interior(exp.n)
    vol = _vol(o, exp.n)
    checks = (1, 2, 5, 10, 20, 50, 100, 150, 200)
    done = 0
    worst = 0.0
    try:
        for step in checks:
            k = step - done
            exact.integrate(k)
            fast.integrate(k)
            o.integrate(k)
            done = step
            ref = o.E[sl]
            got = exact.get_state()[sl]
            assert np.array_equal(got, ref), (step, max_rel(got, ref))
            rel = max_rel(fast.get_state()[sl], ref)
            worst = max(worst, rel)
            assert rel <= FP64_STEP_TOL, (step, rel)
        b, _ = exact.diagnose(fields=False)
        bf, _ = fast.diagnose(fields=False)
        bo = o.diagnose()
        # the sums run over 4.2 M cells in another order than the oracle's
        # sequential loops: compared to 1e-13 of the budget's scale (the
        # z-end boundary flux, for one, nearly cancels under reflection)
        sums = [k for k in bo if k in ("eint", "mflint") or k.startswith("bfl")]
        scale = sum(abs(bo[k]) for k in sums)
        for k in sums:
            assert abs(b[k] - bo[k]) <= 1e-12 * max(abs(bo[k]), 1e-300) + 1e-13 * scale, (k, b[k], bo[k])
        assert abs(b["residual"]) <= 1e-12 * scale
        assert abs(bf["residual"]) <= 1e-12 * scale
        e_ref = float(np.sum(o.E[sl] * vol))
        e_exact = float(np.sum(exact.E[sl] * vol))
        e_fast = float(np.sum(fast.E[sl] * vol))
        assert e_exact == e_ref
        assert abs(e_fast - e_ref) <= 1e-12 * abs(e_ref)
        print("packet 8x8x16x16^3, 200 steps: split bit-identical at %s; fast within %.2e (L-inf), energy %.3e (rel); "
              "residual %.2e of %.2e" % (checks, worst, abs(e_fast - e_ref) / abs(e_ref), b["residual"], scale))
    finally:
        exact.close()
        fast.close()


@pytest.mark.parametrize("name", ["shear_mini", "shear_open", "ragged", "section_2d", "column_1d"])
def test_budget_matches_diagnose(name):
    exp, m, o = _pair(name)
    try:
        m.integrate(2)
        o.integrate(2)
        b, f = m.diagnose()
        bo = o.diagnose()
        sl3 = interior(exp.n[:3])
        for k in ("E_int", "meanfl_int", "diss_ks", "diss_ke", "diss_ls", "diss_le", "diss_ms", "diss_me"):
            assert np.array_equal(f[k][sl3], getattr(o, k)[sl3]), k
        for k in ("mfl_max", "umax", "vmax", "wmax", "kmax", "lmax", "mmax",
                  "cfl_x", "cfl_y", "cfl_z", "cfl_k", "cfl_l", "cfl_m"):
            assert b[k] == bo[k], (k, b[k], bo[k])
        sums = [k for k in b if k in ("eint", "mflint") or k.startswith("bfl")]
        scale = sum(abs(bo[k]) for k in sums) or 1.0
        for k in sums:
            assert abs(b[k] - bo[k]) <= 1e-12 * max(abs(bo[k]), 1e-300) + 1e-15 * scale, (k, b[k], bo[k])
        assert abs(b["residual"]) <= 1e-12 * scale
    finally:
        m.close()


@pytest.mark.parametrize("direct", [True, False], ids=["direct", "staged"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_integrate_host_is_a_drop_in(direct, precision):
    """the host-array step, with the GPU moving the padded array itself or
    through pinned staging, matches the oracle (binary64: bit for bit) and
    leaves the ghost cells alone"""
    exp, m, o = _pair("shear_mini", precision)
    try:
        m.set_host_access(direct)
        ghost_before = m.E.copy()
        m.integrate_host()
        m.integrate_host()
        o.integrate(2)
        sl = interior(exp.n)
        if precision == "fp64":
            assert np.array_equal(m.E[sl], o.E[sl])
        else:
            assert max_rel(m.E[sl], o.E[sl]) < 1e-5
        mask = np.ones(m.E.shape, bool)
        mask[sl] = False
        assert np.array_equal(m.E[mask], ghost_before[mask])   # ghosts untouched
    finally:
        m.close()


def test_host_paths_agree():
    """direct and staged host-array moves give identical states"""
    exp = configs.shear_mini(n=(8, 6, 8, 6, 6, 8))
    outs = []
    for direct in (True, False):
        m = configs.build_model(exp, "fp32")
        m.set_host_access(direct)
        m.set_state()
        m.integrate(3)
        outs.append(m.get_state().copy())
        m.close()
    assert np.array_equal(outs[0], outs[1])


def test_call_order_errors():
    from raytracer_3d_gb300 import Model, _lib
    m = Model(4, 4, 4, 4, 4, 4, dt=1.0)
    try:
        with pytest.raises(_lib.RtError):
            m._check(m._lib.rt_integrate(m.handle, 1), "rt_integrate")
        b = _lib.RtBudget()
        rc = m._lib.rt_diagnose(m.handle, ctypes.byref(b), *([None] * 8))
        assert rc == -5
    finally:
        m.close()


def test_launch_count_and_memory_are_reported():
    exp, m, o = _pair("shear_mini")
    try:
        n0 = m.launch_count()
        m.integrate(3)
        assert m.launch_count() - n0 == 3
        assert m.device_bytes() >= 2 * exp.cells * 8
    finally:
        m.close()


def _energy(E, o, n):
    vol = np.ones(n)
    for a in range(6):
        shp = [1] * 6
        shp[a] = n[a]
        vol = vol * o.grid["xyzklm"[a]]["dt"][ONX:ONX + n[a]].reshape(shp)
    return float(np.sum(E * vol))


def test_fp32_schedules_agree():
    """the schedule never changes the binary32 result"""
    exp = configs.shear_mini(n=(8, 6, 8, 6, 6, 8))
    outs = {}
    for sched in SCHEDULES:
        m = configs.build_model(exp, "fp32")
        m.set_tuning(*sched)
        m.integrate(5)
        outs[sched] = m.get_state().copy()
        m.close()
    first = outs[SCHEDULES[0]]
    for sched, o in outs.items():
        if sched[0] == "cell":
            # the cell kernel may contract multiply-adds differently
            assert max_rel(o, first) < 1e-6
        else:
            assert np.array_equal(o, first), sched


@pytest.mark.parametrize("n", [(32, 32, 4, 4, 2, 6), (24, 16, 6, 4, 6, 10), (16, 8, 5, 2, 4, 6),
                               (20, 12, 4, 2, 4, 6), (64, 64, 4, 2, 2, 2)])
@pytest.mark.parametrize("tuning", [("w3", 4, 128, 1), ("w3", 4, 256, 0), ("w3", 8, 512, 1),
                                    ("w6", 4, 256, 1), ("w6", 8, 512, 0), ("w2z", 4, 256, 1), ("w2z", 8, 512, 0),
                                    ("w2z", 4, 128, 0), ("w2q", 4, 256, 1), ("w2q", 8, 512, 0), ("w2q", 4, 128, 0)],
                         ids=lambda t: "%s-b%d-t%d-s%d" % t)
def test_fp32_persistent_matches_tma(n, tuning):
    """the persistent kernels (several items per CTA, short last band, up to
    4 cells or rows per thread, x faces passed between lanes, ring of
    stages) give the plane-per-CTA TMA result"""
    exp = configs.shear_mini(n=n)
    outs = []
    for sched in (tuning, ("tma", 8, 512, 0)):
        m = configs.build_model(exp, "fp32")
        m.set_tuning(*sched)
        m.integrate(3)
        outs.append(m.get_state().copy())
        m.close()
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("variant", ["tma", "group", "plane", "w3", "w6", "w2z", "w2q", "cell"])
def test_fp32_form_against_fp64_oracle(variant):
    """binary32 state/fluxes/velocities with binary64 coefficients: error
    after 200 steps of the all-axes shear case, both from the initial state
    rounded to binary32 (the input both forms hold exactly).  On this small
    field (1.1e5 cells) the unbiased rounding noise of the binary32 update
    is itself of order 1e-9 over 200 steps, so the drift is held to 1e-9 or
    4 standard deviations of that noise, whichever is larger."""
    exp = configs.shear_mini(n=(8, 6, 8, 6, 6, 8))
    m = configs.build_model(exp, "fp32")
    m.set_tuning(variant)
    o = build_oracle(exp)
    sl = interior(exp.n)
    o.E[sl] = o.E[sl].astype(np.float32).astype(np.float64)
    try:
        assert m.dt == o.dt
        m.integrate(200)
        o.integrate(200)
        m.get_state()
        ref = o.E[sl]
        got = m.E[sl]
        l2 = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        linf = max_rel(got, ref)
        drift = abs(_energy(got, o, exp.n) - _energy(ref, o, exp.n)) / abs(_energy(ref, o, exp.n))
        noise = rounding_noise_bound(ref, vol_widths(o, exp.n), 200)
        print("fp32 vs fp64 oracle after 200 steps: L2 %.3e Linf %.3e energy %.3e (noise allowance %.2e)"
              % (l2, linf, drift, noise))
        assert l2 <= 1e-5
        assert linf <= 1e-4
        assert drift <= max(1e-9, noise)
    finally:
        m.close()


@pytest.mark.parametrize("variant", ["tma", "group", "w2z", "w3", "w6"])
def test_fp32_stretched_against_fp64_oracle(variant):
    """binary32 form on non-uniform grids (per-cell 1/d and dt/2d tables):
    error after 100 steps of the stretched all-axes case, 8x8 planes and 256
    threads so that every listed kernel takes it."""
    exp = configs.stretched_mini(n=(8, 8, 8, 6, 6, 8))
    m = configs.build_model(exp, "fp32")
    m.set_tuning(variant, 8, 256)
    o = build_oracle(exp)
    sl = interior(exp.n)
    try:
        m.integrate(100)
        o.integrate(100)
        m.get_state()
        ref, got = o.E[sl], m.E[sl]
        l2 = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        assert l2 <= 1e-5, l2
        assert max_rel(got, ref) <= 1e-4
    finally:
        m.close()


def test_fp32_budget_residual():
    exp = configs.shear_mini()
    m = configs.build_model(exp, "fp32")
    try:
        m.integrate(3)
        b, f = m.diagnose()
        scale = abs(b["eint"]) + abs(b["mflint"]) + sum(abs(b[k]) for k in b if k.startswith("bfl"))
        assert abs(b["residual"]) <= 1e-5 * scale
    finally:
        m.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_interior_state_matches_padded(precision):
    """a model without the padded host array (interior state in the
    handle's precision) steps exactly like the padded one"""
    exp = configs.shear_mini(n=(8, 6, 8, 6, 6, 8))
    a = configs.build_model(exp, precision)
    b = configs.build_model(exp, precision, padded=False)
    try:
        a.integrate(4)
        b.integrate(4)
        ref = a.get_state()[interior(exp.n)]
        got = b.get_state()
        assert got.shape == tuple(exp.n)
        assert got.dtype == (np.float64 if precision == "fp64" else np.float32)
        assert np.array_equal(got.astype(np.float64), ref)
    finally:
        a.close()
        b.close()
