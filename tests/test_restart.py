"""CPU checks of the restart files (for_src/restart.f90:2-93): the record
layout of gfortran's unformatted sequential files, both byte orders,
subrecords, and the checks read_restart makes."""
import os

import numpy as np
import pytest

from harness import ONX, build_oracle, configs
from raytracer_3d_gb300 import restart


def _arrays(n, seed=0):
    rng = np.random.default_rng(seed)
    shape = tuple(x + 2 * ONX for x in n)
    return [np.asfortranarray(rng.standard_normal(shape)) for _ in range(3)]


def _markers(raw, order="<"):
    """walk the file: [(lead, trail, payload bytes)]"""
    out, pos = [], 0
    mk = np.dtype(order + "i4")
    while pos < len(raw):
        lead = int(np.frombuffer(raw[pos:pos + 4], dtype=mk)[0])
        size = abs(lead)
        trail = int(np.frombuffer(raw[pos + 4 + size:pos + 8 + size], dtype=mk)[0])
        out.append((lead, trail, raw[pos + 4:pos + 4 + size]))
        pos += 8 + size
    return out


def test_file_name():
    assert restart.restart_filename(0) == "restart_pe=000000000.dta"
    assert restart.restart_filename(12) == "restart_pe=000000012.dta"


def test_record_layout_little_endian(tmp_path):
    n = (3, 2, 4, 2, 2, 4)
    E, dE, mf = _arrays(n)
    p = str(tmp_path / "r.dta")
    restart.write_arrays(p, n, 17, E, dE, mf)
    raw = open(p, "rb").read()
    recs = _markers(raw)
    assert [r[0] for r in recs] == [28, 24, 24, 3 * E.size * 8]
    assert all(r[0] == r[1] for r in recs)
    assert list(np.frombuffer(recs[0][2], "<i4")) == list(n) + [17]
    assert list(np.frombuffer(recs[1][2], "<i4")) == [1, 3, 1, 2, 1, 4]
    assert list(np.frombuffer(recs[2][2], "<i4")) == [1, 2, 1, 2, 1, 4]
    vals = np.frombuffer(recs[3][2], "<f8")
    assert np.array_equal(vals[:E.size], E.ravel(order="F"))             # Fortran order, E first
    assert np.array_equal(vals[2 * E.size:], mf.ravel(order="F"))
    assert len(raw) == 4 * 8 + 28 + 24 + 24 + 3 * E.size * 8


@pytest.mark.parametrize("order", ["<", ">"])
def test_round_trip_and_byte_order_detection(tmp_path, order):
    n = (2, 3, 2, 4, 1, 2)
    arrs = _arrays(n, 1)
    p = str(tmp_path / "r.dta")
    restart.write_arrays(p, n, 123456, *arrs, byteorder=order)
    dims, itt, *back = restart.read_arrays(p, n=n)
    assert dims == n and itt == 123456
    for a, b in zip(arrs, back):
        assert np.array_equal(a, b) and b.flags.f_contiguous


def test_subrecords(tmp_path):
    """records longer than the subrecord limit: leading marker negated while
    more follow, trailing marker negated after the first"""
    n = (2, 2, 2, 2, 2, 2)
    arrs = _arrays(n, 2)
    p = str(tmp_path / "r.dta")
    restart.write_arrays(p, n, 5, *arrs, max_subrecord=1000)
    recs = _markers(open(p, "rb").read())
    state = recs[3:]
    total = 3 * arrs[0].size * 8
    assert sum(abs(r[0]) for r in state) == total
    assert state[0][0] == -1000 and state[0][1] == 1000
    assert all(r[0] == -1000 and r[1] == -1000 for r in state[1:-1])
    assert state[-1][0] == total - 1000 * (len(state) - 1) and state[-1][1] == -state[-1][0]
    _, itt, *back = restart.read_arrays(p)
    assert itt == 5 and all(np.array_equal(a, b) for a, b in zip(arrs, back))


def test_read_checks(tmp_path):
    n = (2, 2, 2, 2, 2, 2)
    arrs = _arrays(n, 3)
    p = str(tmp_path / "r.dta")
    restart.write_arrays(p, n, 1, *arrs)
    with pytest.raises(ValueError):                      # restart.f90:66-72
        restart.read_arrays(p, n=(2, 2, 2, 2, 2, 4))
    raw = open(p, "rb").read()
    q = str(tmp_path / "t.dta")
    open(q, "wb").write(raw[:-20])
    with pytest.raises(ValueError):
        restart.read_arrays(q)
    # a PE range of another decomposition (restart.f90:77-85)
    bad = bytearray(raw)
    off = 8 + 28 + 4 + 4                                 # record 2, xe_pe
    bad[off:off + 4] = np.array([1], "<i4").tobytes()
    open(q, "wb").write(bytes(bad))
    with pytest.raises(ValueError):
        restart.read_arrays(q)
    with pytest.raises(ValueError):
        restart.write_arrays(q, n, 1, arrs[0][:-1], arrs[1], arrs[2])


def test_oracle_state_round_trip(tmp_path):
    """the three module arrays of the oracle after a step survive the file"""
    exp = configs.shear_mini()
    o = build_oracle(exp)
    o.integrate(2)
    p = str(tmp_path / restart.restart_filename())
    restart.write_arrays(p, exp.n, 2, o.E, o.dE, o.meanfl)
    dims, itt, E, dE, mf = restart.read_arrays(p, n=exp.n)
    assert itt == 2
    assert np.array_equal(E, o.E) and np.array_equal(dE, o.dE) and np.array_equal(mf, o.meanfl)
    assert os.path.getsize(p) == 4 * 8 + 28 + 48 + 3 * o.E.size * 8
