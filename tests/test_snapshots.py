"""CPU checks of the NetCDF snapshot files (netcdf_io_3D.f90, netcdf_io_6D.f90,
diagnose.f90:331-536) written from the oracle's module arrays: the schema
(dimensions, variables, attributes, CDF-2) and the values read back."""
import numpy as np
import pytest

from harness import ONX, build_oracle, configs, interior
from raytracer_3d_gb300 import snapshots

netcdf = pytest.importorskip("scipy.io").netcdf_file


@pytest.fixture(scope="module")
def run():
    exp = configs.shear_mini(n=(6, 5, 4, 4, 2, 6))
    o = build_oracle(exp)
    o.integrate(2)
    return exp, o


def _write(tmp_path, exp, o, snaps=2):
    p3, p6 = str(tmp_path / "snap3D.cdf"), str(tmp_path / "snap6D.cdf")
    snapshots.init_snap3d(p3, o.grid, exp.n, o.Nsqr, o.U, o.V, exp.f0, exp.fixed)
    om_i, om_e = snapshots.dispersion(o.grid, exp.n, o.Nsqr, o.U, o.V, exp.f0, exp.sign_of_omega_i)
    vel = [getattr(o, v) for v in snapshots.VELOCITIES]
    snapshots.init_snap6d(p6, o.grid, exp.n, vel, om_i, om_e)
    sl = interior(exp.n)
    for s in range(snaps):
        b = o.diagnose()
        fields = {"E_int": o.E_int, "meanfl_int": o.meanfl_int}
        fields.update({k: getattr(o, k) for k in snapshots.DISS})
        assert snapshots.append_snap3d(p3, 100.0 * (s + 1), fields, b) == s + 1
        assert snapshots.append_snap6d(p6, 100.0 * (s + 1), o.E[sl], o.meanfl[sl]) == s + 1
    return p3, p6


def test_dispersion_matches_the_oracle(run):
    exp, o = run
    om_i, om_e = snapshots.dispersion(o.grid, exp.n, o.Nsqr, o.U, o.V, exp.f0, exp.sign_of_omega_i)
    sl = interior(exp.n)
    assert np.array_equal(om_i, o.omega_i[sl]) and np.array_equal(om_e, o.omega_e[sl])


def test_snap3d_schema_and_values(run, tmp_path):
    exp, o = run
    p3, _ = _write(tmp_path, exp, o)
    raw = open(p3, "rb").read(4)
    assert raw == b"CDF\x02"                                      # NF_64BIT_OFFSET
    with netcdf(p3, "r", mmap=False) as f:
        nx, ny, nz = exp.n[:3]
        assert {k: f.dimensions[k] for k in ("xt", "xu", "yt", "yu", "zt", "zu")} == \
            {"xt": nx, "xu": nx, "yt": ny, "yu": ny, "zt": nz, "zu": nz}
        assert f.dimensions["Time"] is None and f.variables["Time"].shape == (2,)
        names = list(f.variables)
        fixed = [k for k in names if "Time" not in f.variables[k].dimensions]
        recs = [k for k in names if "Time" in f.variables[k].dimensions]
        # (the writer orders variables within the file itself; readers use names)
        assert set(fixed) == {"xt", "xu", "yt", "yu", "zt", "zu", "Nsqr", "U", "V"}
        assert set(recs) == set(["Time", "E", "meanfl"] + list(snapshots.DISS) +
                                ["bflux_" + b for b in snapshots.BFLUX] + ["mflint"])
        assert f.variables["E"].dimensions == ("Time", "zt", "yt", "xt")
        assert f.variables["Time"].time_origin == b"01-JAN-1900 00:00:00"
        assert f.variables["E"].long_name == b"energy density".ljust(24)
        assert f.variables["E"].units == b"m^2/s^2".ljust(16)
        assert f.variables["bflux_xs"].long_name == b"Energy flux across min x"
        assert f.f0 == exp.f0 and f.k_fixed == exp.fixed[0]
        sl3 = interior(exp.n[:3])
        assert np.array_equal(f.variables["E"][1], o.E_int[sl3].T)
        assert np.array_equal(f.variables["diss_me"][0], o.diss_me[sl3].T)
        assert np.array_equal(f.variables["Nsqr"][:], o.Nsqr[sl3].T)
        assert np.array_equal(f.variables["zu"][:], o.grid["z"]["u"][ONX:ONX + nz])
        b = o.diagnose()
        assert f.variables["bflux_ke"][1] == b["bfl_ke"] and f.variables["mflint"][0] == b["mflint"]
        assert list(f.variables["Time"][:]) == [100.0, 200.0]


def test_snap6d_schema_and_values(run, tmp_path):
    exp, o = run
    _, p6 = _write(tmp_path, exp, o, snaps=1)
    with netcdf(p6, "r", mmap=False) as f:
        for ax, k in zip("xyzklm", exp.n):
            assert f.dimensions[ax + "t"] == k and f.dimensions[ax + "u"] == k
        assert f.variables["xdot"].dimensions == ("mt", "lt", "kt", "zt", "yt", "xu")
        assert f.variables["mdot"].dimensions == ("mu", "lt", "kt", "zt", "yt", "xt")
        assert f.variables["dkt"].dimensions == ("ku",)
        assert f.variables["E"].dimensions == ("Time", "mt", "lt", "kt", "zt", "yt", "xt")
        assert f.variables["kdot"].long_name == b"hor. wavenr. change".ljust(24)
        sl = interior(exp.n)
        assert np.array_equal(f.variables["E"][0], o.E[sl].T)
        assert np.array_equal(f.variables["meanfl"][0], o.meanfl[sl].T)
        assert np.array_equal(f.variables["zdot"][:], o.zdot[sl].T)
        assert np.array_equal(f.variables["omega_e"][:], o.omega_e[sl].T)
        assert np.array_equal(f.variables["dmt"][:], o.grid["m"]["dt"][ONX:ONX + exp.n[5]])
