"""The C-ABI library builds, loads without a GPU and exports every entry
point declared in include/fall3d_gpu.h (no compute calls here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "fall3d_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(f3d_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from fall3d_gb300 import build

    path = build.build()
    lib = ctypes.CDLL(path)
    names = _declared()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_mirror_fails_loudly_without_library(tmp_path, monkeypatch):
    import fall3d_gb300 as F

    monkeypatch.setattr(F, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(F, "_lib", None)
    with pytest.raises(ImportError):
        F.load()


def test_version_string():
    from fall3d_gb300 import build
    import fall3d_gb300 as F

    build.build()
    assert "sm_103a" in F.version()


def test_ctypes_signatures_match_the_header():
    """The Python mirror declares every entry point with the header's
    argument count, by-value scalars with their C type and pointers as
    pointers (a wrong count or a by-value double passed as an int would
    corrupt the call silently)."""
    import ctypes as C

    import fall3d_gb300 as F
    from fall3d_gb300 import build

    build.build()
    lib = F.load()
    txt = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "fall3d_gpu.h")).read(), flags=re.S)
    scalar = {"int": C.c_int, "double": C.c_double, "long long": C.c_longlong, "float": C.c_float}
    bad = []
    for _, name, args in re.findall(r"^(int|long long|const char\*)\s+(f3d_\w+)\s*\(([^;]*?)\);", txt,
                                    flags=re.M | re.S):
        a = " ".join(args.split())
        params = [] if a in ("", "void") else [p.replace("const ", "").strip() for p in a.split(",")]
        at = getattr(lib, name).argtypes
        if at is None or len(at) != len(params):
            bad.append((name, "count", None if at is None else len(at), len(params)))
            continue
        for i, (p, t) in enumerate(zip(params, at)):
            base = " ".join(p.replace("*", " ").split()[:-1])
            if "*" in p:
                ok = t in (C.c_void_p, C.c_char_p) or (isinstance(t, type) and issubclass(t, C._Pointer))
            else:
                ok = t is scalar.get(base)
            if not ok:
                bad.append((name, i, p, t))
    assert not bad, bad
