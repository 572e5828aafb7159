"""BOLA's routine signatures (alexlovric/bola v0.1.2, src/*.rs) over device
buffers.

Matrices and vectors are CUDA torch tensors used as flat column-major
storage, exactly as BOLA takes `*mut f64` / `&mut [f64]`: element (i, j) of a
matrix with leading dimension lda lives at flat index i + j*lda.  Scalars,
sizes and character flags are plain Python values.  Each call runs on the
current torch CUDA stream and, like BOLA, returns only once the result is
ready.  Errors that BOLA returns as Err(String) raise BolaError with BOLA's
message.
"""
import ctypes

import torch

from . import _lib

NB = 32  # BOLA's block size for getrf/potrf (src/getrf.rs:11, src/potrf.rs:8)


class BolaError(RuntimeError):
    """An error BOLA reports as Err(String); str(e) is BOLA's message."""


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("device buffers only (pass CUDA tensors)")
    return ctypes.c_void_p(t.data_ptr())


def _ch(c):
    return c.encode() if isinstance(c, str) else bytes([c])


def _check(status, what):
    if status != 0:
        msg = _lib.load().bola_last_error().decode(errors="replace")
        raise BolaError(f"{what} failed with status {status}{': ' + msg if msg and status <= -1000 else ''}")


def _sync():
    torch.cuda.current_stream().synchronize()


def set_simd_lanes(lanes):
    """Reproduce BOLA's aarch64/NEON (2) or x86_64/AVX2 (4) rounding."""
    old = _lib.load().bola_set_simd_lanes(int(lanes))
    if old < 0:
        raise ValueError("lanes must be 2 or 4")
    return old


def get_simd_lanes():
    return _lib.load().bola_get_simd_lanes()


# ---- Level 1 ---------------------------------------------------------------

def idamax(n, x):
    """src/idamax.rs:23 — 0-based index of max |x|."""
    out = torch.empty(1, dtype=torch.int64, device=x.device)
    _check(_lib.load().bola_idamax(n, _ptr(x), _ptr(out), _stream()), "idamax")
    return int(out.item())


def scal(n, alpha, x, incx=1):
    """src/scal.rs:45"""
    _check(_lib.load().bola_dscal(n, alpha, _ptr(x), incx, _stream()), "scal")
    _sync()


def ger(m, n, alpha, x, y, ldy, a, lda):
    """src/ger.rs:28"""
    _check(_lib.load().bola_dger(m, n, alpha, _ptr(x), _ptr(y), ldy, _ptr(a), lda, _stream()), "ger")
    _sync()


def dot_product(n, x, incx, y, incy):
    """src/utilities.rs:22"""
    out = torch.empty(1, dtype=torch.float64, device=x.device)
    _check(_lib.load().bola_ddot(n, _ptr(x), incx, _ptr(y), incy, _ptr(out), _stream()), "dot_product")
    return float(out.item())


def daxpy(n, alpha, x, incx, y, incy):
    """src/utilities.rs:107"""
    _check(_lib.load().bola_daxpy(n, alpha, _ptr(x), incx, _ptr(y), incy, _stream()), "daxpy")
    _sync()


def laswp(n, a, lda, k1, k2, ipiv, incx):
    """src/laswp.rs:22 — ipiv is a CUDA int32 tensor."""
    _check(_lib.load().bola_dlaswp(n, _ptr(a), lda, k1, k2, _ptr(ipiv), incx, _stream()), "laswp")
    _sync()


# ---- BLAS 3 ----------------------------------------------------------------

def gemm(transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
    """src/gemm.rs:88"""
    _check(_lib.load().bola_dgemm(_ch(transa), _ch(transb), m, n, k, alpha, _ptr(a), lda, _ptr(b), ldb,
                                   beta, _ptr(c), ldc, _stream()), "gemm")
    _sync()


def trsm(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb):
    """src/trsm.rs:33"""
    _check(_lib.load().bola_dtrsm(_ch(side), _ch(uplo), _ch(transa), _ch(diag), m, n, alpha, _ptr(a), lda,
                                   _ptr(b), ldb, _stream()), "trsm")
    _sync()


def syrk(uplo, trans, n, k, alpha, a, lda, beta, c, ldc):
    """src/syrk.rs:17"""
    _check(_lib.load().bola_dsyrk(_ch(uplo), _ch(trans), n, k, alpha, _ptr(a), lda, beta, _ptr(c), ldc,
                                   _stream()), "syrk")
    _sync()


# ---- LAPACK ------------------------------------------------------------------

INFO_WAIT_EXPIRED = -2000  # BOLA_INFO_WAIT_EXPIRED


def _bola_local_column(info, min_mn):
    # BOLA's messages number the failing column inside the 32-wide block that
    # failed once the matrix is blocked (getrf2 / potrf2 see only that block).
    return info if min_mn <= NB else (info - 1) % NB + 1


def _run_info(fn, *args):
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    status = fn(*args, _ptr(info), _stream())
    return status, info


def getrf(m, n, a, lda, ipiv):
    """src/getrf.rs:37 — LU with partial pivoting; ipiv is CUDA int32."""
    status, info = _run_info(_lib.load().bola_dgetrf, m, n, _ptr(a), lda, _ptr(ipiv))
    if status == -4:
        raise BolaError(f"Argument 4 to getrf had an illegal value of {lda}")
    _check(status, "getrf")
    v = int(info.item())
    if v == INFO_WAIT_EXPIRED:
        raise RuntimeError("getrf: a panel's bounded wait on another CTA expired")
    if v > 0:
        raise BolaError(f"Matrix is singular. The pivot in column {_bola_local_column(v, min(m, n))} is zero.")
    return None


def getrf2(m, n, a, lda, ipiv):
    """src/getrf2.rs:39 — recursive LU."""
    status, info = _run_info(_lib.load().bola_dgetrf2, m, n, _ptr(a), lda, _ptr(ipiv))
    if status == -4:
        raise BolaError(f"Argument 4 to getrf2 had an illegal value of {lda}")
    _check(status, "getrf2")
    v = int(info.item())
    if v == INFO_WAIT_EXPIRED:
        raise RuntimeError("getrf2: a panel's bounded wait on another CTA expired")
    if v > 0:
        raise BolaError(f"Matrix is singular. The pivot in column {v} is zero.")
    return None


def potrf(uplo, n, a, lda):
    """src/potrf.rs:101 — Cholesky."""
    status, info = _run_info(_lib.load().bola_dpotrf, _ch(uplo), n, _ptr(a), lda)
    if status == -1:
        raise BolaError("Argument 1 to potrf had an illegal value")
    if status == -4:
        raise BolaError("Argument 4 to potrf had an illegal value")
    _check(status, "potrf")
    v = int(info.item())
    if v > 0:
        raise BolaError(f"Matrix is not positive-definite. Failure at column {_bola_local_column(v, n)}.")
    return None


def potrf2(uplo, n, a, lda):
    """src/potrf2.rs:25 — recursive Cholesky."""
    status, info = _run_info(_lib.load().bola_dpotrf2, _ch(uplo), n, _ptr(a), lda)
    _check(status, "potrf2")
    v = int(info.item())
    if v > 0:
        raise BolaError(f"Matrix is not positive-definite. Failure at column {v}.")
    return None


def getrs(n, nrhs, lu, lda, ipiv, b, ldb):
    """laswp + unit-lower + upper trsm with getrf's factors."""
    _check(_lib.load().bola_dgetrs(n, nrhs, _ptr(lu), lda, _ptr(ipiv), _ptr(b), ldb, _stream()), "getrs")
    _sync()


def potrs(uplo, n, nrhs, fac, lda, b, ldb):
    """Two triangular solves with potrf's factor."""
    _check(_lib.load().bola_dpotrs(_ch(uplo), n, nrhs, _ptr(fac), lda, _ptr(b), ldb, _stream()), "potrs")
    _sync()


# ---- device-time profiler (BOLA's `profiling` feature, src/profiling.rs) ----

def profile_enable(on=True):
    return bool(_lib.load().bola_profile_enable(1 if on else 0))


def profile_reset():
    _check(_lib.load().bola_profile_reset(), "profile_reset")


def profile_read():
    """{name: {"calls", "ms", "flops", "bytes"}} accumulated since the last reset."""
    L = _lib.load()
    n = L.bola_profile_count()
    if n < 0:
        _check(n, "profile_count")
    out = {}
    for i in range(n):
        name = ctypes.create_string_buffer(64)
        calls, launches = ctypes.c_int64(), ctypes.c_int64()
        ms, fl, by = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _check(L.bola_profile_read(i, name, 64, ctypes.byref(calls), ctypes.byref(launches), ctypes.byref(ms),
                                   ctypes.byref(fl), ctypes.byref(by)), "profile_read")
        out[name.value.decode()] = {"calls": calls.value, "launches": launches.value, "ms": ms.value,
                                    "flops": fl.value, "bytes": by.value}
    return out


def measure_cluster_exchange(csize, nbytes):
    """Microseconds of one all-to-all exchange round among `csize` cluster CTAs
    of `nbytes` each (bola_measure_cluster_exchange)."""
    v = ctypes.c_double(0.0)
    _check(_lib.load().bola_measure_cluster_exchange(int(csize), int(nbytes), ctypes.byref(v)),
           "measure_cluster_exchange")
    return v.value


def measure_fp64_peak():
    """FP64 DFMA throughput of this device in GFLOP/s (bola_measure_fp64_peak)."""
    v = ctypes.c_double()
    _check(_lib.load().bola_measure_fp64_peak(ctypes.byref(v)), "measure_fp64_peak")
    return v.value


def print_profile(prof=None):
    """Report in the shape of BOLA's print_profile (src/profiling.rs:70-115)."""
    prof = profile_read() if prof is None else prof
    if not prof:
        print("no profile data")
        return
    total = max(v["ms"] for v in prof.values())
    print(f"{'routine':<20}{'calls':>8}{'ms total':>12}{'us/call':>12}{'GFLOP/s':>12}{'% of max':>10}")
    for name, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"]):
        gf = v["flops"] / (v["ms"] * 1e6) if v["ms"] > 0 else 0.0
        print(f"{name:<20}{v['calls']:>8}{v['ms']:>12.3f}{1e3 * v['ms'] / max(v['calls'], 1):>12.1f}"
              f"{gf:>12.1f}{100.0 * v['ms'] / total:>9.1f}%")
