"""ctypes binding of the CPU restatement of BOLA (``oracle/bola_oracle.c``).

TEST INFRASTRUCTURE ONLY.  Only the test-suite, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` may import this module; the product
library (``bola_gb300``) never does.  All arrays are numpy, column-major
(Fortran order) float64, ipiv int32 1-based, exactly as BOLA takes them.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_d = ctypes.c_double
_i64 = ctypes.c_int64
_i32 = ctypes.c_int32
_c = ctypes.c_char
_p = ctypes.c_void_p


def build():
    """Compile the restatement with its Makefile (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_SO):
            build()
        L = ctypes.CDLL(_SO)
        sig = {
            "oracle_set_lanes": (None, [ctypes.c_int]),
            "oracle_get_lanes": (ctypes.c_int, []),
            "oracle_set_threads": (None, [ctypes.c_int]),
            "oracle_get_threads": (ctypes.c_int, []),
            "oracle_idamax": (_i64, [_i64, _p]),
            "oracle_scal": (None, [_i64, _d, _p, _i64]),
            "oracle_ger": (None, [_i64, _i64, _d, _p, _p, _i64, _p, _i64]),
            "oracle_dot_product": (_d, [_i64, _p, _i64, _p, _i64]),
            "oracle_daxpy": (None, [_i64, _d, _p, _i64, _p, _i64]),
            "oracle_gemm": (None, [_c, _c, _i64, _i64, _i64, _d, _p, _i64, _p, _i64, _d, _p, _i64]),
            "oracle_trsm": (None, [_c, _c, _c, _c, _i64, _i64, _d, _p, _i64, _p, _i64]),
            "oracle_syrk": (None, [_c, _c, _i64, _i64, _d, _p, _i64, _d, _p, _i64]),
            "oracle_laswp": (None, [_i64, _p, _i64, _i32, _i32, _p, _i32]),
            "oracle_getrf": (ctypes.c_int, [_i64, _i64, _p, _i64, _p]),
            "oracle_getrf2": (ctypes.c_int, [_i64, _i64, _p, _i64, _p]),
            "oracle_potrf": (ctypes.c_int, [_c, _i64, _p, _i64]),
            "oracle_potrf2": (ctypes.c_int, [_c, _i64, _p, _i64]),
            "oracle_set_pivot_margins": (None, [_p, _i64]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _ch(c):
    return c.encode() if isinstance(c, str) else c


def set_lanes(lanes):
    lib().oracle_set_lanes(int(lanes))


def get_lanes():
    return lib().oracle_get_lanes()


def set_threads(t):
    lib().oracle_set_threads(int(t))


def get_threads():
    return lib().oracle_get_threads()


def _check(a, dtype=np.float64):
    assert a.dtype == dtype, a.dtype
    assert a.flags["F_CONTIGUOUS"] or a.ndim == 1, "column-major arrays only"
    return a


def idamax(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    return int(lib().oracle_idamax(x.size, _ptr(x)))


def scal(n, alpha, x, incx=1):
    _check(x)
    lib().oracle_scal(n, alpha, _ptr(x), incx)


def ger(m, n, alpha, x, y, ldy, a, lda):
    lib().oracle_ger(m, n, alpha, _ptr(_check(x)), _ptr(_check(y)), ldy, _ptr(_check(a)), lda)


def dot_product(n, x, incx, y, incy):
    return lib().oracle_dot_product(n, _ptr(_check(x)), incx, _ptr(_check(y)), incy)


def daxpy(n, alpha, x, incx, y, incy):
    lib().oracle_daxpy(n, alpha, _ptr(_check(x)), incx, _ptr(_check(y)), incy)


def gemm(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
    lib().oracle_gemm(_ch(ta), _ch(tb), m, n, k, alpha, _ptr(_check(a)), lda, _ptr(_check(b)), ldb,
                      beta, _ptr(_check(c)), ldc)


def trsm(side, uplo, ta, diag, m, n, alpha, a, lda, b, ldb):
    lib().oracle_trsm(_ch(side), _ch(uplo), _ch(ta), _ch(diag), m, n, alpha, _ptr(_check(a)), lda,
                      _ptr(_check(b)), ldb)


def syrk(uplo, trans, n, k, alpha, a, lda, beta, c, ldc):
    lib().oracle_syrk(_ch(uplo), _ch(trans), n, k, alpha, _ptr(_check(a)), lda, beta,
                      _ptr(_check(c)), ldc)


def laswp(n, a, lda, k1, k2, ipiv, incx):
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    lib().oracle_laswp(n, _ptr(_check(a)), lda, k1, k2, _ptr(ipiv), incx)


def getrf(m, n, a, lda, ipiv):
    """Returns 0, -4 (bad lda) or the 1-based global column of a zero pivot."""
    _check(ipiv, np.int32)
    return int(lib().oracle_getrf(m, n, _ptr(_check(a)), lda, _ptr(ipiv)))


def getrf2(m, n, a, lda, ipiv):
    _check(ipiv, np.int32)
    return int(lib().oracle_getrf2(m, n, _ptr(_check(a)), lda, _ptr(ipiv)))


def potrf(uplo, n, a, lda):
    return int(lib().oracle_potrf(_ch(uplo), n, _ptr(_check(a)), lda))


def potrf2(uplo, n, a, lda):
    return int(lib().oracle_potrf2(_ch(uplo), n, _ptr(_check(a)), lda))


def getrf_with_margins(a, ipiv):
    """getrf on a square/rectangular array; also returns the per-column
    relative gap between the two largest pivot candidates."""
    m, n = a.shape
    margins = np.ones(min(m, n), dtype=np.float64)
    lib().oracle_set_pivot_margins(_ptr(margins), margins.size)
    try:
        info = getrf(m, n, a, max(m, 1), ipiv)
    finally:
        lib().oracle_set_pivot_margins(None, 0)
    return info, margins


def solve_lu(a, b):
    """BOLA composite LU solve (getrf, laswp on B, unit-lower then upper
    trsm).  a (n x n) and b (n x nrhs) are overwritten; returns (info, ipiv)."""
    n = a.shape[0]
    nrhs = b.shape[1]
    ipiv = np.zeros(n, dtype=np.int32)
    info = getrf(n, n, a, n, ipiv)
    if info:
        return info, ipiv
    laswp(nrhs, b, n, 1, n, ipiv, 1)
    trsm("L", "L", "N", "U", n, nrhs, 1.0, a, n, b, n)
    trsm("L", "U", "N", "N", n, nrhs, 1.0, a, n, b, n)
    return 0, ipiv


def solve_chol(a, b):
    """BOLA composite SPD solve: potrf('L'), then L and L^T solves."""
    n = a.shape[0]
    nrhs = b.shape[1]
    info = potrf("L", n, a, n)
    if info:
        return info
    trsm("L", "L", "N", "N", n, nrhs, 1.0, a, n, b, n)
    trsm("L", "L", "T", "N", n, nrhs, 1.0, a, n, b, n)
    return 0
