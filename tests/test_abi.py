"""The C-ABI library builds, loads and exports every entry point the public
header declares (no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(mbqc_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def libpath():
    from mentpy_gb300 import build

    return build.build()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "mbqc_sv_forward" in names and "mbqc_plan_create" in names


def test_library_exports_declared_symbols(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(libpath):
    from mentpy_gb300 import _native

    assert set(declared_symbols()) == set(_native.exported_symbols())
    assert _native.lib().mbqc_abi_version() == 1
