"""The headline workload at its own size: n = 8192, 16 right-hand sides,
A = Q1 diag(sigma) Q2 with sigma geometric from 1 to 1/kappa (Q from the QR
of seeded Gaussian matrices), solved by bola_dgesv_mixed as the benchmark
solves it (3xTF32 factor, GMRES-IR, escalation to the FP64-accurate factor,
FP64 fallback).  Each answer must reach backward error 1e-14, measured here
in FP64 independently of the solver, and its forward error against the FP64
oracle's solution (BOLA's getrf + laswp + trsm(L,L,N,U) + trsm(L,U,N,N) on the
host cores) must stay within c kappa u (u = 2^-53): two solutions with
backward errors e1, e2 differ by about kappa_inf (e1 + e2), and the 1e-14
target is 90u; c = 1000 allows kappa_inf to exceed the 2-norm kappa by a
factor of 5."""
import ctypes

import numpy as np
import pytest
import torch

from bola_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

N, NRHS = 8192, 16
C_FWD = 1000.0


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.fixture(scope="module")
def factors():
    g1 = torch.from_numpy(wl.gaussian_matrix(N, N, seed=3, stream="q1")).cuda()
    g2 = torch.from_numpy(wl.gaussian_matrix(N, N, seed=3, stream="q2")).cuda()
    q1, _ = torch.linalg.qr(g1)
    del g1
    q2, _ = torch.linalg.qr(g2)
    del g2
    xt = torch.from_numpy(wl.uniform_matrix(N, NRHS, seed=3, lo=-1.0, hi=1.0, stream="x")).cuda()
    return q1, q2, xt


@pytest.mark.parametrize("kappa", [1e2, 1e6, 1e10])
def test_config3_solve_vs_oracle(oracle_lib, factors, kappa):
    from bola_gb300 import _lib
    q1, q2, xt = factors
    sigma = torch.logspace(0.0, -np.log10(kappa), N, dtype=torch.float64, device="cuda")
    A = (q1 * sigma) @ q2
    B = A @ xt
    Af = A.t().contiguous().reshape(-1)
    bf = B.t().contiguous().reshape(-1)
    x = torch.zeros(N * NRHS, dtype=torch.float64, device="cuda")
    L = _lib.load()
    opts, info = _lib.MixedOpts(2, 30, 1e-14, 1, 1, 1), _lib.MixedInfo()
    st = L.bola_dgesv_mixed(N, NRHS, _p(Af), N, _p(bf), N, _p(x), N, ctypes.byref(opts), ctypes.byref(info),
                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, L.bola_last_error()
    X = x.reshape(NRHS, N).t()
    R = B - A @ X
    den = A.abs().sum(1).max() * X.abs().max(0).values + B.abs().max(0).values
    e1 = float((R.abs().max(0).values / den).max())
    assert e1 <= 1e-14 and info.backward_error <= 1e-14, (e1, info.backward_error)
    if kappa <= 1e6:
        assert info.path in (0, 1)  # refined on the 3xTF32 factor, no escalation
    A_np = np.asfortranarray(A.cpu().numpy())
    b_np = np.asfortranarray(B.cpu().numpy())
    del A, B, R
    assert oracle_lib.solve_lu(A_np, b_np)[0] == 0
    fwd = np.abs(X.cpu().numpy() - b_np).max() / np.abs(b_np).max()
    assert fwd <= C_FWD * kappa * 2.0 ** -53, (fwd, C_FWD * kappa * 2.0 ** -53)
