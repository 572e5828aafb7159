"""The low-precision LU of the mixed solver on its own (bola_sgetrf_mixed):
64-column panels whose pivots are chosen by tournament over 8-column groups,
tcgen05 trailing updates.  Pivots differ from column-by-column partial
pivoting, so the checks are the factorisation's own properties, in FP64 on
the host: P W = L U to the accuracy of the update kind, ipiv a valid LAPACK
interchange list, and the multipliers bounded (growth of tournament
pivoting)."""
import ctypes

import numpy as np
import pytest
import torch

from bola_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

# |P W - L U| / (|L| |U|)-scale bound per update kind: bf16 operands (2^-8),
# tf32 (2^-11), 3xTF32 (about FP32 accuracy)
TOL = {0: 2e-2, 1: 3e-3, 2: 3e-5}


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def factor(W, n, kind):
    from bola_gb300 import _lib
    L = _lib.load()
    ipiv = torch.zeros(n, dtype=torch.int32, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = L.bola_sgetrf_mixed(kind, n, _p(W), n, _p(ipiv), _p(info),
                             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, L.bola_last_error()
    return ipiv.cpu().numpy(), int(info.item())


def check(A, n, kind):
    W = torch.from_numpy(A.astype(np.float32).ravel(order="F").copy()).cuda()
    ipiv, info = factor(W, n, kind)
    assert info == 0
    assert np.all(ipiv >= np.arange(1, n + 1)) and np.all(ipiv <= n), "ipiv is not a LAPACK interchange list"
    F = W.cpu().numpy().reshape(n, n, order="F").astype(np.float64)
    Lm = np.tril(F, -1) + np.eye(n)
    Um = np.triu(F)
    PA = A.astype(np.float32).astype(np.float64).copy()
    for j in range(n):
        p = ipiv[j] - 1
        if p != j:
            PA[[j, p]] = PA[[p, j]]
    res = np.abs(PA - Lm @ Um).max() / (np.abs(Lm).max() * np.abs(Um).max() * np.sqrt(n))
    return res, np.abs(np.tril(F, -1)).max(), np.abs(Um).max() / np.abs(A).max()


def gepp_growth(A):
    """max|U| / max|A| of column-by-column partial pivoting (LAPACK's getrf via SciPy)."""
    sl = pytest.importorskip("scipy.linalg")
    _, _, U = sl.lu(A)
    return np.abs(U).max() / np.abs(A).max()


@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("n", [64, 200, 1000, 2048])
def test_tournament_lu_factors(kind, n):
    A = wl.uniform_matrix(n, n, seed=21 + n, lo=-1.0, hi=1.0)
    res, lmax, growth = check(A, n, kind)
    assert res <= TOL[kind], res
    assert lmax <= 8.0, lmax  # partial pivoting would give 1; tournament pivoting stays within a few
    # tournament pivoting's growth stays within a small factor of partial
    # pivoting's on the same matrix (about 70 for these at n = 1000, 2048)
    assert growth <= 3.0 * gepp_growth(A), (growth, gepp_growth(A))


def test_tournament_lu_ragged_sizes_and_ties():
    # sizes that leave partial 8-column groups and a short last panel; integer
    # entries make exact ties in the pivot searches (lowest row wins)
    for n in (1, 7, 9, 63, 65, 129, 333):
        rng = np.random.default_rng(n)
        A = rng.integers(-3, 4, (n, n)).astype(np.float64) + 8.0 * np.eye(n)
        res, lmax, _ = check(A, n, 2)
        assert res <= TOL[2], (n, res)
        assert lmax <= 8.0, (n, lmax)


def test_tournament_lu_zero_column_reports_info():
    n = 300
    A = wl.uniform_matrix(n, n, seed=5, lo=-1.0, hi=1.0)
    A[:, 77] = 0.0  # column 78 (1-based) has no nonzero pivot left
    W = torch.from_numpy(A.astype(np.float32).ravel(order="F").copy()).cuda()
    _, info = factor(W, n, 2)
    assert info == 78


@pytest.mark.parametrize("n,ldw", [(1001, 1004), (333, 336), (2050, 2056)])
def test_tournament_lu_padded_leading_dimension(n, ldw):
    """ldw > n, a multiple of 4 (the panel's float4 write-back runs) with n
    not one (ragged last runs); the padding rows keep their values."""
    from bola_gb300 import _lib
    L = _lib.load()
    A = wl.uniform_matrix(n, n, seed=n, lo=-1.0, hi=1.0)
    buf = np.full((ldw, n), 7.25, dtype=np.float32)
    buf[:n] = A.astype(np.float32)
    W = torch.from_numpy(buf.ravel(order="F").copy()).cuda()
    ipiv = torch.zeros(n, dtype=torch.int32, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = L.bola_sgetrf_mixed(2, n, _p(W), ldw, _p(ipiv), _p(info),
                             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0 and int(info.item()) == 0
    out = W.cpu().numpy().reshape(ldw, n, order="F")
    assert np.all(out[n:] == 7.25)
    # the same factors as with ldw = n
    W2 = torch.from_numpy(A.astype(np.float32).ravel(order="F").copy()).cuda()
    ipiv2, _ = factor(W2, n, 2)
    assert np.array_equal(ipiv.cpu().numpy(), ipiv2)
    assert np.array_equal(out[:n], W2.cpu().numpy().reshape(n, n, order="F"))
