"""Binary32 form against the binary64 form on the jet workload: the
binary64 GPU form is bit-identical to the oracle (test_gpu_parity.py), so
it is the reference for long runs the CPU oracle cannot reach in a test.
Reports relative L2 and L-infinity differences of E and the drift of the
total energy sum(E*vol) after 1000 steps of jet_large at 16^6, and holds
them to the binary32 form's bounds: L2 <= 1e-5, drift <= 1e-9."""
import numpy as np
import pytest

from harness import configs, interior
from raytracer_3d_gb300.grid import ONX

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()


def _energy(E, m):
    vol = np.ones(m.n)
    for a in range(6):
        shp = [1] * 6
        shp[a] = m.n[a]
        vol = vol * m.grid["xyzklm"[a]]["dt"][ONX:ONX + m.n[a]].reshape(shp)
    return float(np.sum(E * vol))


def test_fp32_jet_1000_steps_against_fp64():
    """both forms start from the initial state rounded to binary32, the
    input both hold exactly"""
    exp = configs.jet_large(n=(16,) * 6)
    m64 = configs.build_model(exp, "fp64")
    m32 = configs.build_model(exp, "fp32")
    try:
        assert m32.dt == m64.dt
        sl = interior(exp.n)
        m64.E[sl] = m64.E[sl].astype(np.float32).astype(np.float64)
        m64.set_state()
        e0 = _energy(m64.E[sl], m64)
        m64.integrate(1000)
        m32.integrate(1000)
        ref = m64.get_state()[sl].copy()
        got = m32.get_state()[sl]
        l2 = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        linf = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
        e64, e32 = _energy(ref, m64), _energy(got, m32)
        drift = abs(e32 - e64) / abs(e64)
        print("jet_large 16^6, 1000 steps: L2 %.3e  Linf %.3e  energy fp32 vs fp64 %.3e  "
              "(fp64 energy change over the run %.3e)" % (l2, linf, drift, abs(e64 - e0) / abs(e0)))
        assert np.isfinite(got).all()
        assert l2 <= 1e-5
        assert linf <= 1e-4
        assert drift <= 1e-9
    finally:
        m64.close()
        m32.close()
