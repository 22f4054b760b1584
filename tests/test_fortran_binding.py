"""The Fortran binding (fortran/rt_gpu.f90) against the C header, as text
(no Fortran compiler exists here): every bind(C) name is a function that
include/rt_gb300.h declares, and the bind(C) derived types list the fields
of the C structs in the same order with matching kinds."""
import os
import re

from harness import ROOT

F90 = os.path.join(ROOT, "fortran", "rt_gpu.f90")
HDR = os.path.join(ROOT, "include", "rt_gb300.h")


def _header():
    return re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)


def test_bound_names_are_declared():
    txt = open(F90).read()
    names = re.findall(r'bind\(C,\s*name="(\w+)"\)', txt)
    assert len(names) >= 20
    hdr = _header()
    for n in names:
        assert re.search(r"\b%s\s*\(" % n, hdr), n


def _c_struct(name):
    m = re.search(r"typedef struct \{([^{}]*)\}\s*%s;" % name, _header())
    assert m, name
    fields = []
    for line in m.group(1).split(";"):
        line = re.sub(r"//.*", "", line).strip()
        if not line:
            continue
        typ = line.split()[0]
        for f in line[len(typ):].split(","):
            fields.append((typ, f.strip()))
    return fields


def _f_type(name):
    m = re.search(r"type, bind\(C\) :: %s\n(.*?)end type %s" % (name, name), open(F90).read(), flags=re.S)
    assert m, name
    fields = []
    for line in m.group(1).strip().splitlines():
        kind, rest = line.split("::")
        typ = "double" if "c_double" in kind else "int"
        fields += [(typ, f.strip()) for f in rest.split(",")]
    return fields


def test_derived_types_match_the_c_structs():
    for name in ("rt_dims", "rt_params", "rt_budget"):
        assert _f_type(name) == _c_struct(name), name
