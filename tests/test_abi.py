"""CPU checks of the C ABI: the library loads, exports every function that
include/rt_gb300.h declares, and rejects bad arguments without touching a
GPU."""
import ctypes
import os
import re

import pytest

from harness import ROOT

HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"^\s*[A-Za-z_][\w\s\*]*?\b(rt_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build_library()
    from raytracer_3d_gb300 import _lib
    return _lib.load()


def test_header_declares_the_path():
    names = declared_functions()
    for n in ("rt_create", "rt_calc_parameter", "rt_integrate", "rt_diagnose", "rt_set_state",
              "rt_get_state", "rt_destroy", "rt_last_error"):
        assert n in names


def test_every_declared_symbol_is_exported(lib):
    for n in declared_functions():
        assert hasattr(lib, n), n


def test_python_binding_covers_header():
    from raytracer_3d_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_argument_validation_without_gpu(lib):
    from raytracer_3d_gb300 import _lib
    h = ctypes.c_void_p()
    par = _lib.RtParams(1.0, 1e-4, 1.0, 1, 1, _lib.RT_FP64)
    bad = [_lib.RtDims(8, 8, 8, 7, 8, 8, 2),     # nk odd (parallel_mpi.f90:17)
           _lib.RtDims(8, 8, 8, 8, 8, 8, 3),     # onx must be 2
           _lib.RtDims(0, 8, 8, 8, 8, 8, 2)]
    for d in bad:
        rc = lib.rt_create(ctypes.byref(d), ctypes.byref(par), ctypes.byref(h))
        assert rc == -1
        assert lib.rt_last_error(None)
    par_bad = _lib.RtParams(-1.0, 1e-4, 1.0, 1, 1, _lib.RT_FP64)
    rc = lib.rt_create(ctypes.byref(_lib.RtDims(8, 8, 8, 8, 8, 8, 2)), ctypes.byref(par_bad), ctypes.byref(h))
    assert rc == -1


def test_version_string(lib):
    assert b"sm_103a" in lib.rt_version()


def test_timers_and_selftest_reject_null_arguments(lib):
    assert lib.rt_tic(None, b"integrate") == -1
    assert lib.rt_toc(None, b"integrate") == -1
    secs = ctypes.c_double()
    assert lib.rt_timing_secs(None, b"integrate", ctypes.byref(secs), None) == -1
    assert lib.rt_selftest_wait_timeout(None, None) == -1
    assert lib.rt_get_tendency(None, None, None) == -1


def test_noalloc_rejects_bad_dims_without_gpu(lib):
    """the allocation-free rate rejects a halo width other than 2 and a
    cell count beyond its fixed scratch, including products that would
    overflow a 64-bit integer (six axes of 65536 = 2^96 cells), before any
    CUDA call"""
    from raytracer_3d_gb300 import _lib
    P = ctypes.POINTER(ctypes.c_double)
    null6 = (P * 6)()
    out = ctypes.cast(1, P)
    for dims, word in ((_lib.RtDims(8, 8, 8, 8, 8, 8, 3), b"onx"),
                       (_lib.RtDims(*([65536] * 6), 2), b"exceed"),
                       (_lib.RtDims(2, 2, 2, 2, 2, 2 ** 30, 2), b"exceed")):
        rc = lib.rt_max_rate_noalloc(ctypes.byref(dims), null6, null6, null6, out, None)
        assert rc == -1
        assert word in lib.rt_noalloc_last_error()
