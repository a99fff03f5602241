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
