"""The oracle and the GPU library against the committed golden fixtures."""
import hashlib

import numpy as np
import pytest

from golden_cases import GPU_NAMES, NAMES, load
from harness import build_oracle, configs, interior

DIAG3 = ("E_int", "meanfl_int", "diss_ks", "diss_ke", "diss_ls", "diss_le", "diss_ms", "diss_me")


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name):
    exp, meta, arrs = load(name)
    o = build_oracle(exp)
    assert o.dt == meta["dt"]
    sl = interior(exp.n)
    for s in range(meta["steps"]):
        o.integrate(1)
        assert _sha(o.E[sl]) == meta["step_sha256"][s], (name, s)
    assert np.array_equal(o.E[sl], arrs["E"])
    b = o.diagnose()
    for k, v in meta["budget"].items():
        assert b[k] == v, k
    sl3 = interior(exp.n[:3])
    for k in DIAG3:
        assert np.array_equal(getattr(o, k)[sl3], arrs[k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("name", GPU_NAMES)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gpu_against_golden(name, precision):
    import __graft_entry__ as g
    g.build()
    exp, meta, arrs = load(name)
    m = configs.build_model(exp, precision)
    sl = interior(exp.n)
    try:
        if precision == "fp64":
            assert m.dt == meta["dt"]
            for s in range(meta["steps"]):
                m.integrate(1)
                assert _sha(m.get_state()[sl]) == meta["step_sha256"][s], (name, s)
            b, f = m.diagnose()
            sl3 = interior(exp.n[:3])
            for k in DIAG3:
                assert np.array_equal(f[k][sl3], arrs[k]), k
        else:
            m.integrate(meta["steps"])
            got = m.get_state()[sl]
            ref = arrs["E"]
            assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref)
    finally:
        m.close()
