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


def test_a_c_host_compiles_and_links_against_the_library(tmp_path):
    """The header is plain C (C99, -pedantic, no warnings) and a C program
    that takes the address of every declared entry point links against the
    library and runs (no compute call: it only prints the library version
    string's length) -- what a C or Fortran host does when it binds the ABI."""
    import shutil
    import subprocess

    from fall3d_gb300 import build

    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    lib = build.build()
    names = _declared()
    src = tmp_path / "host.c"
    src.write_text(
        '#include <stdio.h>\n#include <string.h>\n#include "fall3d_gpu.h"\n'
        "typedef void (*fn)(void);\n"
        "int main(void) {\n"
        f"  fn table[] = {{ {', '.join(f'(fn){n}' for n in names)} }};\n"
        "  printf(\"%d %d\\n\", (int)(sizeof table / sizeof table[0]), (int)strlen(f3d_version()) > 0);\n"
        "  return 0;\n}\n")
    exe = tmp_path / "host"
    libdir = os.path.dirname(lib)
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-Wno-cast-function-type",
                        "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe), "-L", libdir,
                        "-l:" + os.path.basename(lib), "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split() == [str(len(names)), "1"]


def test_the_product_does_not_use_the_oracle():
    """The library and its Python mirror neither import, load nor name a
    path of oracle/ (the oracle is test infrastructure): no import of an
    oracle module, no oracle/ path and no liboracle in the package, the
    header or the CUDA sources."""
    pkg = os.path.join(ROOT, "fall3d_gb300")
    files = [os.path.join(dp, f) for dp, _, fs in os.walk(pkg) for f in fs
             if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")) and "_build" not in dp]
    files += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    pat = re.compile(r"import\s+(oracle_lib|ref_driver|ref_translate)|from\s+(oracle|ref_driver|ref_translate)\b|"
                     r"oracle/|liboracle|f3d_oracle|oracle_lib")
    hits = []
    for f in files:
        for i, line in enumerate(open(f, errors="replace"), 1):
            if pat.search(line):
                hits.append(f"{os.path.relpath(f, ROOT)}:{i}: {line.strip()}")
    assert not hits, hits
