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


def _c_params():
    """name -> list of (by_value, kind) per parameter of the header's
    functions; kind is the C base type (int, double, long long, char,
    void, or the struct / handle name)."""
    src = open(os.path.join(ROOT, "include", "fall3d_gpu.h")).read()
    body = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for _, name, args in re.findall(r"^(int|long long|const char\*)\s+(f3d_\w+)\s*\(([^;]*?)\);", body,
                                    flags=re.M | re.S):
        a = " ".join(args.split())
        params = []
        if a not in ("", "void"):
            for p in a.split(","):
                p = p.replace("const ", "").strip()
                stars = p.count("*")
                base = p.replace("*", " ").split()
                base = " ".join(base[:-1])  # drop the parameter name
                params.append((stars, base))
        out[name] = params
    return out


def _f90_params():
    """name -> list of (by_value, fortran type) per dummy argument, in the
    order of the function statement."""
    text = re.sub(r"&\s*\n\s*", "", _f90())
    out = {}
    for m in re.finditer(r"function (f3d_\w+)\(([^)]*)\) bind\(C, name=\"\w+\"\)\n(.*?)end function \1", text,
                         flags=re.S):
        name, args, block = m.group(1), m.group(2), m.group(3)
        decl = {}
        for line in block.splitlines():
            line = line.split("!")[0].strip()
            if "::" not in line:
                continue
            spec, names = [x.strip() for x in line.split("::")]
            typ = spec.split(",")[0].strip()
            attrs = [x.strip() for x in spec.split(",")[1:]]
            for nm in names.split(","):
                nm = nm.strip()
                arr = nm.endswith("(*)")
                decl[nm.replace("(*)", "").lower()] = ("value" in attrs, typ, arr)
        out[name] = [decl[a.strip().lower()] for a in args.split(",") if a.strip()]
    return out


# C base type -> the Fortran type of a value or of the pointee
_KIND = {"int": "integer(c_int)", "double": "real(c_double)", "float": "real(c_float)", "long long": "integer(c_long_long)",
         "char": "character(kind=c_char)"}


def test_every_argument_is_passed_as_the_header_declares():
    """By value in C <=> VALUE in Fortran, with the same kind; a pointer to a
    scalar or array <=> a by-reference dummy of the pointee's kind (or an
    opaque type(c_ptr), value); the context and batch / server handles
    <=> type(c_ptr), value; a handle's address (f3d_ctx** and the like) <=>
    type(c_ptr) by reference; a struct pointer <=> the bind(C) derived type
    by reference."""
    c, f = _c_params(), _f90_params()
    assert set(c) == set(f)
    handles = {"f3d_ctx", "f3d_batch", "f3d_server"}
    bad = []
    for name, cps in c.items():
        for i, ((stars, base), (val, typ, arr)) in enumerate(zip(cps, f[name])):
            if stars == 0:
                ok = val and typ == _KIND.get(base)
            elif base in handles or base == "void":
                ok = (stars == 1 and val and typ == "type(c_ptr)") or (stars == 2 and not val and typ == "type(c_ptr)")
            elif base.startswith("f3d_"):
                ok = not val and typ == f"type({base})"
            else:
                ok = (not val and typ == _KIND.get(base)) or (val and typ == "type(c_ptr)")
            if not ok:
                bad.append((name, i, stars, base, val, typ))
    assert not bad, bad
