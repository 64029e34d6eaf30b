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
    assert _native.lib().mbqc_abi_version() == 2


def _header_constants():
    src = open(os.path.join(ROOT, "include", "mbqc_gb300.h")).read()
    out = {}
    for name, val in re.findall(r"#define\s+(MBQC_[A-Z0-9_]+)\s+\(?(-?(?:0x[0-9a-fA-F]+|\d+))u?\)?", src):
        out[name] = int(val, 0)
    return out


def test_python_constants_match_header():
    """Status codes, flags and plane codes seen by the Python layer are the
    header's values."""
    from mentpy_gb300 import _native
    from mentpy_gb300.plan import DEAD, PLANE_CODES

    h = _header_constants()
    for name in dir(_native):
        if re.fullmatch(r"MBQC_(OK|E_[A-Z]+|F_[A-Z_]+)", name):
            assert h[name] == getattr(_native, name), name
    for plane, code in PLANE_CODES.items():
        assert h[f"MBQC_PLANE_{plane}"] == code
    assert h["MBQC_STEP_DEAD"] == DEAD
    assert {n for n in h if n.startswith("MBQC_F_")} <= {n for n in dir(_native) if n.startswith("MBQC_F_")}
