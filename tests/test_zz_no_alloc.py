"""rt_max_rate_noalloc: the CFL-rate reduction for callers that cannot
allocate device memory (a framework that owns all allocations, a frozen
graph or real-time loop, no out-of-memory failure allowed mid-run).  Its
scratch is a fixed array inside the library, so it is called here on
caller-owned device arrays and compared with rt_max_rate, twice in a row
(the second call sees the scratch left behind by the first)."""
import ctypes

import numpy as np
import pytest

from harness import ONX, configs

pytestmark = pytest.mark.gpu


def _device_copy(torch, arr):
    t = torch.from_numpy(np.ascontiguousarray(arr.ravel(order="F"))).to("cuda")
    return t


@pytest.mark.parametrize("name", ["shear", "packet"])
def test_noalloc_rate_matches_handle_rate(name):
    import __graft_entry__ as g
    g.build()
    torch = pytest.importorskip("torch")
    from raytracer_3d_gb300 import _lib
    exp = configs.shear_mini(n=(7, 5, 6, 4, 6, 4)) if name == "shear" else configs.packet_small()
    m = configs.build_model(exp, "fp64")
    try:
        ref = m.max_rate()
        n = exp.n
        keep = []
        vel, vlo, dg = [], [], []
        for a in range(6):
            f = m.get_field(a)                             # padded, faces 0..n along a
            inner = [slice(ONX, ONX + k) for k in n]
            right = f[tuple(inner)]                        # faces 1..n = right faces
            lo = list(inner)
            lo[a] = slice(ONX - 1, ONX)                    # face 0 plane
            plane = f[tuple(lo)]
            tr, tp = _device_copy(torch, right), _device_copy(torch, plane)
            td = _device_copy(torch, np.ascontiguousarray(m.grid["xyzklm"[a]]["dt"]))
            keep += [tr, tp, td]
            vel.append(tr.data_ptr())
            vlo.append(tp.data_ptr())
            dg.append(td.data_ptr())
        P = ctypes.POINTER(ctypes.c_double)
        arr = lambda ptrs: (P * 6)(*[ctypes.cast(p, P) for p in ptrs])  # noqa: E731
        out = torch.zeros(1, dtype=torch.float64, device="cuda")
        dims = _lib.RtDims(*n, ONX)
        lib = _lib.load()
        stream = torch.cuda.current_stream().cuda_stream
        for _ in range(2):
            out.fill_(-1.0)
            rc = lib.rt_max_rate_noalloc(ctypes.byref(dims), arr(vel), arr(vlo), arr(dg),
                                         ctypes.cast(out.data_ptr(), P), ctypes.c_void_p(stream))
            assert rc == 0, lib.rt_noalloc_last_error()
            torch.cuda.synchronize()
            got = float(out.item())
            assert got == ref, (got, ref)       # a maximum: exact in any order
    finally:
        m.close()


def test_noalloc_rejects_oversized_field():
    import __graft_entry__ as g
    g.build()
    from raytracer_3d_gb300 import _lib
    lib = _lib.load()
    P = ctypes.POINTER(ctypes.c_double)
    null6 = (P * 6)()
    dims = _lib.RtDims(64, 64, 64, 64, 64, 64, ONX)     # 2^36 cells
    rc = lib.rt_max_rate_noalloc(ctypes.byref(dims), null6, null6, null6, ctypes.cast(1, P), None)
    assert rc == -1
    assert b"exceed" in lib.rt_noalloc_last_error()
