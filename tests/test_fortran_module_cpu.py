"""include/fall3d_gpu.f90, the Fortran bind(C) module of the library: every
function declared in include/fall3d_gpu.h has an interface of the same name
with the same number of arguments, and every bind(C) derived type lists the
fields of its C struct in the C order with matching kinds (the ctypes
mirror of fall3d_gb300/_abi.py is the reference for the C layout).  No
Fortran compiler is installed here, so the module is checked by parsing."""
import ctypes as C
import os
import re

from fall3d_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _c_functions():
    src = open(os.path.join(ROOT, "include", "fall3d_gpu.h")).read()
    body = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for _, name, args in re.findall(r"^(int|long long|const char\*)\s+(f3d_\w+)\s*\(([^;]*?)\);", body,
                                    flags=re.M | re.S):
        a = " ".join(args.split())
        out[name] = 0 if a in ("", "void") else len(a.split(","))
    return out


def _f90():
    return open(os.path.join(ROOT, "include", "fall3d_gpu.f90")).read()


def test_every_entry_point_has_an_interface():
    text = re.sub(r"&\s*\n\s*", "", _f90())
    f90 = {}
    for name, args, cname in re.findall(r"function (f3d_\w+)\(([^)]*)\) bind\(C, name=\"(\w+)\"\)", text):
        assert name == cname
        f90[name] = 0 if not args.strip() else len(args.split(","))
    c = _c_functions()
    assert set(f90) == set(c), sorted(set(c) ^ set(f90))
    for name, n in c.items():
        assert f90[name] == n, (name, f90[name], n)


def test_derived_types_match_the_structs():
    text = _f90()
    kinds = {"integer(c_int)": "c_int", "real(c_double)": "c_double", "type(c_ptr)": "ptr"}
    pairs = {"f3d_grid": _abi.F3DGrid, "f3d_met_series": _abi.F3DMetSeries, "f3d_src_series": _abi.F3DSrcSeries,
             "f3d_log_record": _abi.F3DLogRecord, "f3d_gravity_current": _abi.F3DGravityCurrent,
             "f3d_aggregation": _abi.F3DAggregation}
    for tname, struct in pairs.items():
        block = re.search(rf"type, bind\(C\) :: {tname}\n(.*?)end type {tname}", text, flags=re.S).group(1)
        block = re.sub(r"&\s*\n\s*", "", block)
        fields = []
        for line in block.splitlines():
            line = line.split("!")[0].strip()
            if not line:
                continue
            kind, names = [x.strip() for x in line.split("::")]
            fields += [(n.strip().lower(), kinds[kind]) for n in names.split(",")]
        want = []
        for n, ct in struct._fields_:
            k = "c_int" if ct is C.c_int else "c_double" if ct is C.c_double else "ptr"
            want.append((n.lower(), k))
        assert fields == want, (tname, fields, want)


def test_every_constant_is_a_parameter():
    src = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "fall3d_gpu.h")).read(), flags=re.S)
    c = {n: int(v, 0) for n, v in re.findall(r"^#define\s+(F3D_\w+)\s+\(?(-?(?:0x[0-9a-fA-F]+|\d+))\)?\s*$",
                                              src, flags=re.M)}
    f = {n: int(v) for n, v in re.findall(r"integer\(c_int\), parameter :: (F3D_\w+) = (-?\d+)", _f90())}
    assert c, "no constants parsed from the header"
    assert f == c, sorted(set(c.items()) ^ set(f.items()))
