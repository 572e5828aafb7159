"""numpy-facing wrapper of bola_gb300.api with the oracle binding's interface:
arrays are copied to the GPU, the C-ABI routine runs, results are copied back
into the caller's arrays.  Lets one test body drive both implementations."""
import numpy as np
import torch

from bola_gb300 import api


def _dev(a):
    flat = np.asarray(a).ravel(order="F") if np.asarray(a).ndim > 1 else np.asarray(a)
    return torch.from_numpy(np.ascontiguousarray(flat)).cuda()


def _back(arr, t):
    host = t.cpu().numpy()
    if arr.ndim > 1:
        arr[...] = host.reshape(arr.shape, order="F")
    else:
        arr[...] = host


class GpuBackend:
    """Numpy in, numpy out; each call goes through the C ABI."""

    def set_lanes(self, lanes):
        api.set_simd_lanes(lanes)

    def get_lanes(self):
        return api.get_simd_lanes()

    def idamax(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        return api.idamax(x.size, _dev(x))

    def scal(self, n, alpha, x, incx=1):
        t = _dev(x)
        api.scal(n, alpha, t, incx)
        _back(x, t)

    def ger(self, m, n, alpha, x, y, ldy, a, lda):
        ta = _dev(a)
        api.ger(m, n, alpha, _dev(x), _dev(y), ldy, ta, lda)
        _back(a, ta)

    def dot_product(self, n, x, incx, y, incy):
        return api.dot_product(n, _dev(x), incx, _dev(y), incy)

    def daxpy(self, n, alpha, x, incx, y, incy):
        ty = _dev(y)
        api.daxpy(n, alpha, _dev(x), incx, ty, incy)
        _back(y, ty)

    def gemm(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
        tc = _dev(c)
        api.gemm(ta, tb, m, n, k, alpha, _dev(a), lda, _dev(b), ldb, beta, tc, ldc)
        _back(c, tc)

    def trsm(self, side, uplo, ta, diag, m, n, alpha, a, lda, b, ldb):
        tb = _dev(b)
        api.trsm(side, uplo, ta, diag, m, n, alpha, _dev(a), lda, tb, ldb)
        _back(b, tb)

    def syrk(self, uplo, trans, n, k, alpha, a, lda, beta, c, ldc):
        tc = _dev(c)
        api.syrk(uplo, trans, n, k, alpha, _dev(a), lda, beta, tc, ldc)
        _back(c, tc)

    def laswp(self, n, a, lda, k1, k2, ipiv, incx):
        t = _dev(a)
        api.laswp(n, t, lda, k1, k2, _dev(np.asarray(ipiv, dtype=np.int32)), incx)
        _back(a, t)

    def _info_call(self, fn, a, *args):
        t = _dev(a)
        try:
            fn(t, *args)
            info = 0
        except api.BolaError as e:
            info = e
        _back(a, t)
        return info

    def getrf(self, m, n, a, lda, ipiv):
        t, tp = _dev(a), _dev(ipiv)
        info = 0
        try:
            api.getrf(m, n, t, lda, tp)
        except api.BolaError as e:
            info = str(e)
        _back(a, t)
        _back(ipiv, tp)
        return info

    def getrf2(self, m, n, a, lda, ipiv):
        t, tp = _dev(a), _dev(ipiv)
        info = 0
        try:
            api.getrf2(m, n, t, lda, tp)
        except api.BolaError as e:
            info = str(e)
        _back(a, t)
        _back(ipiv, tp)
        return info

    def potrf(self, uplo, n, a, lda):
        t = _dev(a)
        info = 0
        try:
            api.potrf(uplo, n, t, lda)
        except api.BolaError as e:
            info = str(e)
        _back(a, t)
        return info

    def potrf2(self, uplo, n, a, lda):
        t = _dev(a)
        info = 0
        try:
            api.potrf2(uplo, n, t, lda)
        except api.BolaError as e:
            info = str(e)
        _back(a, t)
        return info

    def getrs(self, n, nrhs, lu, lda, ipiv, b, ldb):
        tb = _dev(b)
        api.getrs(n, nrhs, _dev(lu), lda, _dev(np.asarray(ipiv, dtype=np.int32)), tb, ldb)
        _back(b, tb)

    def potrs(self, uplo, n, nrhs, fac, lda, b, ldb):
        tb = _dev(b)
        api.potrs(uplo, n, nrhs, _dev(fac), lda, tb, ldb)
        _back(b, tb)
