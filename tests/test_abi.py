"""The C-ABI library (host-side checks, no GPU): it loads, and it exports
every function include/bola_gb300.h declares, with the ctypes signatures the
Python layer uses.  No compute call is made."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "bola_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bola_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from bola_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from bola_gb300 import build
        build.build()
    return _lib.load()


def test_header_declares_the_bola_routines():
    names = declared_functions()
    for routine in ["gemm", "getrf", "getrf2", "potrf", "potrf2", "trsm", "syrk", "laswp", "idamax", "scal",
                    "ger", "ddot", "daxpy"]:
        assert any(n.endswith(routine) or n == "bola_" + routine or n == "bola_d" + routine for n in names), routine


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(lib):
    from bola_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES), set(declared_functions()) - set(_lib.SIGNATURES)


def test_host_only_entry_points(lib):
    assert lib.bola_version().startswith(b"bola_gb300")
    assert lib.bola_set_simd_lanes(4) == 2
    assert lib.bola_get_simd_lanes() == 4
    assert lib.bola_set_simd_lanes(3) == -1
    assert lib.bola_set_simd_lanes(2) == 4


def test_argument_checks_need_no_device(lib):
    """Illegal arguments are rejected on the host before any CUDA call."""
    null = ctypes.c_void_p(0)
    assert lib.bola_dgetrf(4, 4, null, 3, null, null, null) == -4
    assert lib.bola_dpotrf(b"l", 4, null, 4, null, null) == -1
    assert lib.bola_dpotrf(b"L", 4, null, 3, null, null) == -4
    assert lib.bola_dgemm(b"N", b"N", -1, 2, 2, 1.0, null, 1, null, 2, 0.0, null, 1, null) == -3
    assert lib.bola_dtrsm(b"L", b"L", b"N", b"U", 4, 2, 1.0, null, 3, null, 4, null) == -9
