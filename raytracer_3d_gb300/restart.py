"""Restart files of the reference (for_src/restart.f90:2-93), written and
read by the host.

write_restart writes, as one Fortran unformatted sequential file
'restart_pe=000000000.dta' (restart.f90:8-9; one rank, so pe 0):

  record 1  nx, ny, nz, nk, nl, nm, itt             7 default integers
  record 2  xs_pe, xe_pe, ys_pe, ye_pe, zs_pe, ze_pe 6 default integers
  record 3  ks_pe, ke_pe, ls_pe, le_pe, ms_pe, me_pe 6 default integers
  record 4  E, dE, meanfl                           3 padded 6D real*8 arrays

(restart.f90:15-18) and the formatted file 'ritt' holding itt
(restart.f90:21-26).  The layout is gfortran's: every record is framed by a
4-byte length marker before and after its data; a record longer than
2**31-9 bytes is split into subrecords whose leading marker is negated when
another subrecord follows and whose trailing marker is negated when one
precedes.  Byte order is the machine's (little endian) unless the reference
was built with -fconvert=big-endian (make.inc:11); byteorder ">" writes
that form and the reader detects either.

E comes from rt_get_state, dE and meanfl from rt_get_tendency (the arrays
the last step left behind); before any step they are zero, as the
reference's allocate_main_module leaves them.  Ghost cells are written as
the host arrays hold them; the reference refills them before it reads them
(integrate.f90:14-94).
"""
import os

import numpy as np

from .grid import ONX

MAX_SUBRECORD = 2 ** 31 - 9      # largest subrecord gfortran writes
RESTART_NAME = "restart_pe=%09d.dta"


def restart_filename(pe=0):
    """'restart_pe=' // i9 with blanks replaced by zeros // '.dta' (restart.f90:8-9)"""
    return RESTART_NAME % pe


def _write_record(f, payload, byteorder, max_sub):
    n = len(payload)
    mk = np.dtype(byteorder + "i4")
    if n == 0:
        f.write(np.array([0, 0], dtype=mk).tobytes())
        return
    pos = 0
    while pos < n:
        size = min(max_sub, n - pos)
        more = pos + size < n
        lead = -size if more else size
        trail = -size if pos > 0 else size
        f.write(np.array([lead], dtype=mk).tobytes())
        f.write(payload[pos:pos + size])
        f.write(np.array([trail], dtype=mk).tobytes())
        pos += size


def _read_record(f, byteorder):
    mk = np.dtype(byteorder + "i4")
    parts = []
    first = True
    while True:
        head = f.read(4)
        if len(head) < 4:
            raise ValueError("restart file: truncated record marker")
        lead = int(np.frombuffer(head, dtype=mk)[0])
        size = abs(lead)
        data = f.read(size)
        tail = f.read(4)
        if len(data) < size or len(tail) < 4:
            raise ValueError("restart file: truncated record")
        trail = int(np.frombuffer(tail, dtype=mk)[0])
        if abs(trail) != size or (trail < 0) == first:
            raise ValueError("restart file: record markers %d / %d do not match" % (lead, trail))
        parts.append(data)
        first = False
        if lead >= 0:
            return b"".join(parts)


def _detect_order(path):
    with open(path, "rb") as f:
        head = f.read(4)
    if len(head) < 4:
        raise ValueError("restart file %s is empty" % path)
    for order in ("<", ">"):
        if int(np.frombuffer(head, dtype=np.dtype(order + "i4"))[0]) == 7 * 4:
            return order
    raise ValueError("restart file %s: first record is not 7 integers" % path)


def write_arrays(path, n, itt, E, dE, meanfl, byteorder="<", max_subrecord=MAX_SUBRECORD):
    """Write the four restart records for dims n (one rank: the PE ranges
    are 1..n per axis) and the padded arrays E, dE, meanfl."""
    n = tuple(int(x) for x in n)
    shape = tuple(x + 2 * ONX for x in n)
    ints = np.dtype(byteorder + "i4")
    reals = np.dtype(byteorder + "f8")
    arrays = []
    for name, a in (("E", E), ("dE", dE), ("meanfl", meanfl)):
        a = np.asarray(a)
        if a.shape != shape:
            raise ValueError("%s must have the padded shape %s, got %s" % (name, shape, a.shape))
        arrays.append(np.asarray(a, dtype=reals).tobytes(order="F"))
    with open(path, "wb") as f:
        _write_record(f, np.array(n + (int(itt),), dtype=ints).tobytes(), byteorder, max_subrecord)
        _write_record(f, np.array([1, n[0], 1, n[1], 1, n[2]], dtype=ints).tobytes(), byteorder, max_subrecord)
        _write_record(f, np.array([1, n[3], 1, n[4], 1, n[5]], dtype=ints).tobytes(), byteorder, max_subrecord)
        _write_record(f, b"".join(arrays), byteorder, max_subrecord)


def read_arrays(path, n=None, byteorder=None):
    """Read a restart file; returns (n, itt, E, dE, meanfl) with padded
    Fortran-order arrays.  With n given, the dimensions and the PE ranges
    must match it, as read_restart demands (restart.f90:66-85)."""
    order = byteorder or _detect_order(path)
    ints = np.dtype(order + "i4")
    with open(path, "rb") as f:
        r1 = np.frombuffer(_read_record(f, order), dtype=ints)
        r2 = np.frombuffer(_read_record(f, order), dtype=ints)
        r3 = np.frombuffer(_read_record(f, order), dtype=ints)
        if r1.size != 7 or r2.size != 6 or r3.size != 6:
            raise ValueError("restart file %s: unexpected header records" % path)
        dims = tuple(int(x) for x in r1[:6])
        itt = int(r1[6])
        if n is not None and tuple(n) != dims:
            raise ValueError("restart dimensions %s do not match %s" % (dims, tuple(n)))
        ranges = tuple(int(x) for x in np.concatenate([r2, r3]))
        want = tuple(v for k in dims for v in (1, k))
        if ranges != want:
            raise ValueError("restart PE boundaries %s do not match one rank %s" % (ranges, want))
        shape = tuple(x + 2 * ONX for x in dims)
        cnt = int(np.prod(shape))
        raw = _read_record(f, order)
        if len(raw) != 3 * cnt * 8:
            raise ValueError("restart file %s: state record has %d bytes, expected %d" % (path, len(raw), 3 * cnt * 8))
    vals = np.frombuffer(raw, dtype=np.dtype(order + "f8")).astype(np.float64)
    E, dE, meanfl = (vals[k * cnt:(k + 1) * cnt].reshape(shape, order="F").copy(order="F") for k in range(3))
    return dims, itt, E, dE, meanfl


def write_restart(model, directory=".", itt=None, byteorder="<", pe=0):
    """write_restart (restart.f90:2-32) for a Model: its device state and
    the tendency of its last step.  Returns the restart file's path."""
    E = np.array(model.get_state(), dtype=np.float64, order="F", copy=True)
    if not getattr(model, "padded", True):
        pad = np.zeros(tuple(x + 2 * ONX for x in model.n), order="F")
        pad[tuple(slice(ONX, ONX + k) for k in model.n)] = E
        E = pad
    dE, meanfl = model.get_tendency()
    itt = model.itt if itt is None else int(itt)
    path = os.path.join(directory, restart_filename(pe))
    write_arrays(path, model.n, itt, E, dE, meanfl, byteorder=byteorder)
    with open(os.path.join(directory, "ritt"), "w") as f:
        f.write("%12d\n" % itt)              # list-directed write of one integer
    return path


def read_restart(model, directory=".", pe=0):
    """read_restart (restart.f90:37-93) for a Model: a missing file leaves
    the model as it is and returns None; otherwise the state is uploaded,
    model.itt set, and (itt, dE, meanfl) returned."""
    path = os.path.join(directory, restart_filename(pe))
    if not os.path.exists(path):
        return None
    _, itt, E, dE, meanfl = read_arrays(path, n=model.n)
    sl = tuple(slice(ONX, ONX + k) for k in model.n)
    if getattr(model, "padded", True):
        model.E[...] = E
    else:
        model.E[...] = E[sl].astype(model.E.dtype)
    model.set_state()
    model.itt = itt
    return itt, dE, meanfl
