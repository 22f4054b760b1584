"""The C++ host driver (host/rt_main.cpp, main.f90 over the C ABI) on the
GPU: its run equals the oracle's from the same inputs bit for bit, under
both binary64 schedules, and a run continued from its restart file equals
the uninterrupted run."""
import subprocess

import numpy as np
import pytest

from harness import ONX, build_oracle, interior
from raytracer_3d_gb300.configs import Experiment

pytestmark = pytest.mark.gpu
AXES = "xyzklm"


@pytest.fixture(scope="module")
def driver():
    import __graft_entry__ as g
    g.build()
    from raytracer_3d_gb300 import build
    return build.build_host()


def _run(driver, *args):
    r = subprocess.run([driver] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return r.stdout


def _meta(d):
    out = {}
    for line in (d / "meta.txt").read_text().splitlines():
        k, v = line.split(" = ", 1)
        out[k] = v
    return out


def _bin(d, name):
    return np.fromfile(str(d / (name + ".bin")), dtype="<f8")


def _experiment(d):
    """the driver's run as an experiment for the oracle, from its dump"""
    meta = _meta(d)
    n = tuple(int(x) for x in meta["n"].split())
    P3 = tuple(k + 2 * ONX for k in n[:3])
    P6 = tuple(k + 2 * ONX for k in n)
    dint = [_bin(d, "grid_%s_dt" % ax)[ONX:ONX + n[a]] for a, ax in enumerate(AXES)]

    def background(m):
        m.Nsqr[:] = _bin(d, "Nsqr").reshape(P3, order="F")
        m.U[:] = _bin(d, "U").reshape(P3, order="F")
        m.V[:] = _bin(d, "V").reshape(P3, order="F")

    def initial(m, rng):
        m.E[:] = _bin(d, "E0").reshape(P6, order="F")

    exp = Experiment(meta["name"], n, dint, float(meta["f0"]), background, initial, int(meta["steps"]),
                     dt=float(meta["dt"]), sign_of_omega_i=float(meta["sign"]), upper=meta["upper"] == "1",
                     lower=meta["lower"] == "1", fixed=tuple(float(x) for x in meta["fixed"].split()))
    return exp, meta, _bin(d, "E").reshape(P6, order="F")


@pytest.mark.parametrize("name,steps", [("packet_small", 4), ("column_1d", 6)])
@pytest.mark.parametrize("schedule", ["tma", "split"])
def test_driver_run_equals_the_oracle(driver, tmp_path, name, steps, schedule):
    d = tmp_path / "dump"
    d.mkdir()
    out = _run(driver, name, "--steps", steps, "--snap", 2, "--schedule", schedule, "--dump", d)
    assert "Timing summary" in out and "residual" in out
    exp, meta, E = _experiment(d)
    assert int(meta["itt"]) == steps
    o = build_oracle(exp)
    o.integrate(steps)
    sl = interior(exp.n)
    assert np.array_equal(E[sl], o.E[sl])
    scale = abs(float(meta["eint"])) + abs(float(meta["mflint"])) + 1e-300
    assert abs(float(meta["residual"])) <= 1e-10 * scale


def test_driver_restart_continues_exactly(driver, tmp_path):
    whole, rdir, part = tmp_path / "whole", tmp_path / "restart", tmp_path / "part"
    for p in (whole, rdir, part):
        p.mkdir()
    _run(driver, "column_1d", "--steps", 6, "--dump", whole)
    _run(driver, "column_1d", "--steps", 3, "--restart", rdir)           # no file yet: writes one at itt 3
    assert (rdir / "restart_pe=000000000.dta").exists()
    out = _run(driver, "column_1d", "--steps", 3, "--restart", rdir, "--dump", part)
    assert "reading restart file" in out
    _, mw, Ew = _experiment(whole)
    _, mp, Ep = _experiment(part)
    assert int(mp["itt"]) == 6
    n = tuple(int(x) for x in mw["n"].split())
    sl = interior(n)
    assert np.array_equal(Ew[sl], Ep[sl])
    # the file is readable by the Python host's reader, with the dimensions checked
    from raytracer_3d_gb300 import restart
    dims, itt, E, dE, mf = restart.read_arrays(str(rdir / "restart_pe=000000000.dta"), n=n)
    assert itt == 6 and np.array_equal(E[sl], Ep[sl]) and np.abs(dE[sl]).max() > 0
