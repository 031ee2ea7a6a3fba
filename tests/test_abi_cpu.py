"""C-ABI checks that need no GPU: the library builds for sm_103a, loads, and
exports every function that include/*.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    inc = os.path.join(ROOT, "include")
    for fn in sorted(os.listdir(inc)):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = "\n".join(l for l in text.split("\n") if not l.lstrip().startswith(("typedef", "#")))
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*([a-z][a-z0-9_]*)\s*\(", text, flags=re.M):
            if m.group(1) not in ("typedef",):
                names.append(m.group(1))
    return sorted(set(names))


@pytest.fixture(scope="module")
def libpath():
    from rustpde_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("rbc_create", "rbc_step", "rbc_get_state", "fs_forward", "sv_solve"):
        assert n in names
    assert len(names) >= 40


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"missing exports: {missing}"


def test_python_mirror_binds_every_symbol(libpath):
    import rustpde_gb300 as R
    L = R.lib()
    for n in R._SIGNATURES:
        assert hasattr(L, n)
    assert set(R._SIGNATURES) <= set(declared_functions())


def test_no_cpu_fallback_without_library(tmp_path, monkeypatch):
    import rustpde_gb300 as R
    monkeypatch.setattr(R, "_lib", None)
    monkeypatch.setattr(R, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(RuntimeError):
        R.lib()
