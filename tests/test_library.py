"""CPU checks of the C-ABI library: it builds for sm_103a, loads, and exports
every entry point include/virgpu.h declares (no compute calls)."""
import ctypes
import os
import re

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(REPO, "include", "virgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vg_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_exports_header():
    from vir_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 8
    for s in syms:
        assert hasattr(lib, s), s
    lib.vg_version.restype = ctypes.c_int
    assert lib.vg_version() >= 100


def test_python_bindings_cover_header():
    from vir_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.exported_symbols())


def test_status_strings():
    from vir_gb300 import build
    lib = ctypes.CDLL(build.build())
    lib.vg_status_string.restype = ctypes.c_char_p
    assert lib.vg_status_string(0) == b"ok"
    assert lib.vg_status_string(1) == b"bad argument"


def test_argument_errors_without_gpu():
    """Invalid sizes are rejected on the host before any launch."""
    from vir_gb300 import _lib
    L = _lib.load()
    g = _lib.DD2DGeom(0, 10, 5, 5, 1.0, 0.0, 1.0, 0.0, 0.0, 0)
    st = L.vg_dd2d_fp(ctypes.byref(g), None, None, None, None, None)
    assert st == 1
    assert b"positive" in L.vg_last_error()
