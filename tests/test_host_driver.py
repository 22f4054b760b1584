"""CPU checks of the C++ host driver (raytracer_3d_gb300/host/rt_main.cpp),
the counterpart of for_src/main.f90 over the C ABI: it builds, its host
grids equal the Python host's and the oracle's bit for bit, its
experiments' inputs match the Python definitions, and a failing library
call stops it with halt_stop's exit code 99."""
import os
import subprocess

import numpy as np
import pytest

from harness import ONX, build_oracle, configs
from raytracer_3d_gb300 import grid

AXES = "xyzklm"


@pytest.fixture(scope="module")
def driver():
    import __graft_entry__ as g
    g.build_library()
    from raytracer_3d_gb300 import build
    return build.build_host()


def _dump(driver, tmp_path, name):
    d = tmp_path / name
    d.mkdir()
    r = subprocess.run([driver, name, "--dry", "--dump", str(d)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    return d


def _bin(d, name):
    return np.fromfile(str(d / (name + ".bin")), dtype="<f8")


def test_help(driver):
    r = subprocess.run([driver, "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "packet_small" in r.stdout


@pytest.mark.parametrize("name,make", [("column_1d", lambda: configs.column_1d(fac=1)),
                                       ("packet_small", lambda: configs.packet_small())])
def test_grids_and_inputs_match_the_python_host(driver, tmp_path, name, make):
    d = _dump(driver, tmp_path, name)
    exp = make()
    g = grid.calc_grid(exp.n, exp.d_interior, exp.fixed)
    for a, ax in enumerate(AXES):
        for key in ("t", "u", "dt", "du"):
            assert np.array_equal(_bin(d, "grid_%s_%s" % (ax, key)), g[ax][key]), (ax, key)
    o = build_oracle(exp)
    P3 = tuple(k + 2 * ONX for k in exp.n[:3])
    P6 = tuple(k + 2 * ONX for k in exp.n)
    for f, ref in (("Nsqr", o.Nsqr), ("U", o.U), ("V", o.V)):
        got = _bin(d, f).reshape(P3, order="F")
        # exp / tanh of the C library and of numpy may differ in the last
        # place (1 + tanh cancels where tanh nears -1: absolute tolerance)
        assert np.allclose(got, ref, rtol=1e-15, atol=1e-15 * np.abs(ref).max()), f
    E0 = _bin(d, "E0").reshape(P6, order="F")
    # the packet's noise comes from the driver's own generator (at most 1e-8)
    atol = 1.01e-8 if name == "packet_small" else 1e-15
    assert np.allclose(E0, o.E, rtol=1e-14, atol=atol)
    assert (E0 != 0).sum() == (o.E != 0).sum() or name == "packet_small"


def test_failing_call_stops_with_halt_stop_code(driver, tmp_path):
    """Without a GPU rt_create fails and the driver stops with exit code 99
    (halt_stop, parallel_mpi.f90:223-236); with one it runs the steps."""
    r = subprocess.run([driver, "column_1d", "--steps", "1"], capture_output=True, text=True, timeout=300)
    if r.returncode == 99:
        assert "rt_create" in r.stderr and "aborting" in r.stderr
    else:
        assert r.returncode == 0, r.stderr
        assert "Timing summary" in r.stdout


def test_unknown_arguments_stop_the_run(driver):
    for args in (["nonexistent"], ["column_1d", "--bogus"]):
        r = subprocess.run([driver] + args, capture_output=True, text=True, timeout=60)
        assert r.returncode == 99
