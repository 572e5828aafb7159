"""Mixed-precision SPD solve (bola_dposv_mixed): tensor-core Cholesky of
D A D, FP64 refinement.  Each answer must reach the normwise backward error
target 1e-14; its forward error is checked against the FP64 oracle, BOLA's
own potrf('L') + trsm(L,L,N,N) + trsm(L,L,T,N) solve: two backward-stable
solutions with backward errors e1, e2 differ by at most about
2 kappa (e1 + e2) relative to the solution, so the test requires
    ||x - x_oracle|| / ||x_oracle|| <= c kappa u,  u = 2^-53,  c = 400
(the 1e-14 target is 90u; c covers 2 (90u + u) with a factor 2 of slack).
The factor alone (bola_spotrf_mixed) is checked for L L^T = W."""
import ctypes

import numpy as np
import pytest
import torch

from bola_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

U = 2.0 ** -53
C_FWD = 400.0


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def make_spd(n, nrhs, kappa, seed):
    g = torch.from_numpy(wl.gaussian_matrix(n, n, seed=seed, stream="q1")).cuda()
    q, _ = torch.linalg.qr(g)
    sigma = torch.logspace(0.0, -np.log10(kappa), n, dtype=torch.float64, device="cuda")
    A = (q * sigma) @ q.t()
    A = 0.5 * (A + A.t())
    xt = torch.from_numpy(wl.uniform_matrix(n, nrhs, seed=seed, lo=-1, hi=1, stream="x")).cuda()
    b = A @ xt
    return A.t().contiguous().reshape(-1), b.t().contiguous().reshape(-1)


def posv(A, b, n, nrhs, kind, fallback=1, escalate=1):
    from bola_gb300 import _lib
    L = _lib.load()
    x = torch.zeros(n * nrhs, dtype=torch.float64, device="cuda")
    opts = _lib.MixedOpts(kind, 30, 1e-14, fallback, 1, escalate)
    info = _lib.MixedInfo()
    st = L.bola_dposv_mixed(n, nrhs, _p(A), n, _p(b), n, _p(x), n, ctypes.byref(opts), ctypes.byref(info),
                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, L.bola_last_error()
    return x, info


def berr(A, x, b, n, nrhs):
    Am = A.reshape(n, n).t()
    X = x.reshape(nrhs, n).t()
    B = b.reshape(nrhs, n).t()
    R = B - Am @ X
    den = Am.abs().sum(1).max() * X.abs().max(0).values + B.abs().max(0).values
    return float((R.abs().max(0).values / den).max())


@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("n", [64, 300, 1000])
def test_cholesky_factor(kind, n):
    from bola_gb300 import _lib
    L = _lib.load()
    A, _ = make_spd(n, 1, 1e3, seed=30 + n)
    W0 = A.reshape(n, n).cpu().numpy().astype(np.float32)  # symmetric, so row/column order is moot
    W = torch.from_numpy(W0.ravel(order="F").copy()).cuda()
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = L.bola_spotrf_mixed(kind, n, _p(W), n, _p(info), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, L.bola_last_error()
    assert int(info.item()) == 0
    Lf = np.tril(W.cpu().numpy().reshape(n, n, order="F").astype(np.float64))
    res = np.abs(Lf @ Lf.T - W0.astype(np.float64)).max() / np.abs(W0).max()
    assert res <= {0: 3e-2, 1: 3e-3, 2: 3e-5}[kind], res
    assert np.all(np.diag(Lf) > 0)


def test_cholesky_factor_reports_a_negative_pivot():
    from bola_gb300 import _lib
    L = _lib.load()
    n = 200
    A, _ = make_spd(n, 1, 10.0, seed=5)
    W0 = A.reshape(n, n).cpu().numpy().astype(np.float32)
    W0[130, 130] = -1.0  # not positive definite: the pivot of column 131 cannot be positive
    W = torch.from_numpy(W0.ravel(order="F").copy()).cuda()
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert L.bola_spotrf_mixed(2, n, _p(W), n, _p(info), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
    assert 0 < int(info.item()) <= 131


@pytest.mark.parametrize("kappa", [1e2, 1e6, 1e10])
@pytest.mark.parametrize("n,nrhs", [(257, 3), (1024, 16)])
def test_mixed_cholesky_solve_vs_oracle(oracle_lib, kappa, n, nrhs):
    A, b = make_spd(n, nrhs, kappa, seed=7)
    x, info = posv(A, b, n, nrhs, 2)
    assert info.backward_error <= 1e-14
    e1 = berr(A, x, b, n, nrhs)
    assert e1 <= 1e-14
    assert info.factorization == 1 and info.path in (0, 1, 3), (info.factorization, info.path)
    if kappa <= 1e6:
        assert info.path in (0, 1)  # the 3xTF32 Cholesky refines without escalation
    A_np = A.cpu().numpy().reshape(n, n).T.copy(order="F")
    b_np = b.cpu().numpy().reshape(nrhs, n).T.copy(order="F")
    assert oracle_lib.solve_chol(A_np, b_np) == 0
    X = x.cpu().numpy().reshape(nrhs, n).T
    fwd = np.abs(X - b_np).max() / np.abs(b_np).max()
    assert fwd <= C_FWD * kappa * U, (fwd, C_FWD * kappa * U)


def test_not_spd_falls_back_to_the_mixed_lu():
    n, nrhs = 300, 2
    A, b = make_spd(n, nrhs, 1e2, seed=8)
    Am = A.reshape(n, n)
    Am[100, 100] = -Am[100, 100]  # still symmetric, no longer positive definite
    b = (Am.t() @ torch.ones(n, nrhs, dtype=torch.float64, device="cuda")).t().contiguous().reshape(-1)
    x, info = posv(A, b, n, nrhs, 2)
    assert info.factorization == 0 and info.factor_info > 0
    assert berr(A, x, b, n, nrhs) <= 1e-14


def test_cholesky_solve_matches_lu_solve_quality():
    # the same SPD system through both entry points: both meet the target
    n, nrhs = 1024, 4
    A, b = make_spd(n, nrhs, 1e4, seed=9)
    xc, ic = posv(A, b, n, nrhs, 2)
    from bola_gb300 import _lib
    L = _lib.load()
    xl = torch.zeros_like(xc)
    opts, il = _lib.MixedOpts(2, 30, 1e-14, 1, 1, 1), _lib.MixedInfo()
    assert L.bola_dgesv_mixed(n, nrhs, _p(A), n, _p(b), n, _p(xl), n, ctypes.byref(opts), ctypes.byref(il),
                              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
    assert ic.factorization == 1 and il.factorization == 0
    assert berr(A, xc, b, n, nrhs) <= 1e-14 and berr(A, xl, b, n, nrhs) <= 1e-14
