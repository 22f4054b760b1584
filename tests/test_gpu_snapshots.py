"""NetCDF snapshots written from the GPU library (Snapshots over a Model)
hold the oracle's fields: E, meanfl, the velocities and the wavenumber
integrals bit-identical in binary64, the boundary sums to reordering."""
import numpy as np
import pytest

from harness import build_oracle, configs, interior
from raytracer_3d_gb300 import snapshots

pytestmark = pytest.mark.gpu
netcdf = pytest.importorskip("scipy.io").netcdf_file


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()


def test_snapshots_from_the_gpu(tmp_path):
    exp = configs.shear_mini(n=(6, 5, 4, 4, 2, 6))
    m = configs.build_model(exp, "fp64")
    o = build_oracle(exp)
    try:
        snap = snapshots.Snapshots(m, str(tmp_path))
        for _ in range(2):
            m.integrate(2)
            o.integrate(2)
            snap.write()
        bo = o.diagnose()
        sl, sl3 = interior(exp.n), interior(exp.n[:3])
        with netcdf(snap.path6d, "r", mmap=False) as f:
            assert list(f.variables["Time"][:]) == [2 * m.dt, 4 * m.dt]
            assert np.array_equal(f.variables["E"][1], o.E[sl].T)
            assert np.array_equal(f.variables["meanfl"][1], o.meanfl[sl].T)
            for v in snapshots.VELOCITIES:
                assert np.array_equal(f.variables[v][:], getattr(o, v)[sl].T), v
            assert np.array_equal(f.variables["omega_i"][:], o.omega_i[sl].T)
        with netcdf(snap.path3d, "r", mmap=False) as f:
            assert np.array_equal(f.variables["E"][1], o.E_int[sl3].T)
            assert np.array_equal(f.variables["diss_ks"][1], o.diss_ks[sl3].T)
            scale = sum(abs(bo[k]) for k in bo if k.startswith("bfl")) + abs(bo["mflint"])
            for b in snapshots.BFLUX:
                assert abs(f.variables["bflux_" + b][1] - bo["bfl_" + b]) <= 1e-12 * scale
    finally:
        m.close()
