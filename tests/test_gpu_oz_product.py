"""FP64-accurate products on the tensor cores (bola_dgemv_oz): the residual
r = b - A x and the product A x of the mixed solver's refinement, computed
from exact 8-bit digit planes of A and x.  Checked against the exact product
(binary128 arithmetic on the host: a product of two doubles is exact there)
with the error bound the method guarantees,
    |out - exact| <= 2^-52 n max_j|a_ij| max|x_c| + 2^-51 |(A x)_ic| + 2^-52 |r_ic|
(the digit roundings, the dropped digit pairs and the final FP64 roundings,
with a factor 4 of slack), including heavy cancellation (b = fl(A x)), rows
and columns scaled over many orders of magnitude, ragged sizes, several
blocks of 16 right-hand sides, zeros, and NaN propagation."""
import ctypes

import numpy as np
import pytest
import torch

from bola_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

QUAD = np.finfo(np.longdouble).nmant >= 112


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def oz(A, X, B=None):
    """A (n x n), X (n x k), B (n x k) float64 numpy arrays -> device result."""
    from bola_gb300 import _lib
    L = _lib.load()
    n, k = X.shape
    dA = torch.from_numpy(np.asfortranarray(A).ravel(order="F")).cuda()
    dX = torch.from_numpy(np.asfortranarray(X).ravel(order="F")).cuda()
    dB = torch.from_numpy(np.asfortranarray(B).ravel(order="F")).cuda() if B is not None else None
    out = torch.full((n * k,), 7.0, dtype=torch.float64, device="cuda")
    st = L.bola_dgemv_oz(n, k, _p(dA), n, _p(dX), n, _p(dB), n, _p(out), n,
                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, L.bola_last_error()
    return out.cpu().numpy().reshape(n, k, order="F")


def check(A, X, B=None):
    if not QUAD:
        pytest.skip("needs binary128 long double for the exact reference (aarch64 host)")
    n = A.shape[0]
    got = oz(A, X, B)
    AX = A.astype(np.longdouble) @ X.astype(np.longdouble)
    exact = (B.astype(np.longdouble) - AX) if B is not None else AX
    Mi = np.abs(A).max(axis=1, keepdims=True)
    Xc = np.abs(X).max(axis=0, keepdims=True)
    tol = 2.0 ** -52 * n * Mi * Xc + 2.0 ** -51 * np.abs(AX).astype(np.float64) + \
        2.0 ** -52 * np.abs(exact).astype(np.float64)
    err = np.abs((got.astype(np.longdouble) - exact)).astype(np.float64)
    assert np.all(np.isfinite(got))
    assert np.all(err <= tol), (err / np.maximum(tol, 1e-300)).max()
    return got, exact


@pytest.mark.parametrize("n,k", [(1, 1), (7, 3), (129, 16), (1000, 16), (2048, 20)])
def test_product_exact_to_the_bound(n, k):
    A = wl.uniform_matrix(n, n, seed=40 + n, lo=-1.0, hi=1.0)
    X = wl.uniform_matrix(n, k, seed=41 + n, lo=-1.0, hi=1.0)
    check(A, X)


@pytest.mark.parametrize("n,k", [(513, 4), (1024, 16)])
def test_residual_under_cancellation(n, k):
    # b = fl(A x): the exact residual is at the rounding level of b, and the
    # computed one must resolve it to within the bound (an FP64 DGEMM cannot)
    A = wl.uniform_matrix(n, n, seed=50 + n, lo=-1.0, hi=1.0)
    X = wl.uniform_matrix(n, k, seed=51 + n, lo=-1.0, hi=1.0)
    B = A @ X
    got, exact = check(A, X, B)
    # the residual itself, not just the bound: relative to |b| it is ~1e-16
    assert np.abs(got).max() <= 1e-13 * np.abs(B).max()


def test_rows_and_columns_scaled_over_many_orders():
    n, k = 700, 16
    rng = np.random.default_rng(3)
    A = wl.uniform_matrix(n, n, seed=60, lo=-1.0, hi=1.0) * np.exp2(rng.integers(-300, 300, n))[:, None]
    A *= np.exp2(rng.integers(-20, 20, n))[None, :]  # columns too: rows are far from uniform
    X = wl.uniform_matrix(n, k, seed=61, lo=-1.0, hi=1.0) * np.exp2(rng.integers(-200, 200, k))[None, :]
    check(A, X)
    check(A, X, A @ X)


def test_zeros_and_nonfinite_operands():
    n, k = 300, 5
    A = wl.uniform_matrix(n, n, seed=70, lo=-1.0, hi=1.0)
    X = wl.uniform_matrix(n, k, seed=71, lo=-1.0, hi=1.0)
    A[17, :] = 0.0
    X[:, 2] = 0.0
    got, _ = check(A, X)
    assert np.all(got[17, :] == 0.0) and np.all(got[:, 2] == 0.0)
    X[5, 3] = np.nan
    A2 = A.copy()
    A2[40, 9] = np.inf
    got = oz(A2, X)
    assert np.all(np.isnan(got[:, 3]))          # a NaN in column 3 of x
    assert np.all(np.isnan(got[40, :]))         # an Inf in row 40 of A
    ok = np.ones_like(got, dtype=bool)
    ok[:, 3] = False
    ok[40, :] = False
    assert np.all(np.isfinite(got[ok]))
