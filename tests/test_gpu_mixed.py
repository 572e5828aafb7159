"""Mixed-precision solve (tensor-core LU + FP64 refinement) against the FP64
oracle (BOLA's getrf + trsm solve): every result must reach the normwise
backward error target 1e-14, and its forward error against the oracle's
solution must stay within kappa * 1e-14 (the conditioning bound)."""
import ctypes

import numpy as np
import pytest
import torch

from bola_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def make_system(n, nrhs, kappa, seed):
    g1 = torch.from_numpy(wl.gaussian_matrix(n, n, seed=seed, stream="q1")).cuda()
    g2 = torch.from_numpy(wl.gaussian_matrix(n, n, seed=seed, stream="q2")).cuda()
    q1, _ = torch.linalg.qr(g1)
    q2, _ = torch.linalg.qr(g2)
    sigma = torch.logspace(0.0, -np.log10(kappa), n, dtype=torch.float64, device="cuda")
    A = (q1 * sigma) @ q2
    xt = torch.from_numpy(wl.uniform_matrix(n, nrhs, seed=seed, lo=-1, hi=1, stream="x")).cuda()
    b = A @ xt
    return A.t().contiguous().reshape(-1), b.t().contiguous().reshape(-1)


def solve(A, b, n, nrhs, kind, fallback=1, max_it=30, gmres=1, escalate=0):
    from bola_gb300 import _lib
    L = _lib.load()
    x = torch.zeros(n * nrhs, dtype=torch.float64, device="cuda")
    opts = _lib.MixedOpts(kind, max_it, 1e-14, fallback, gmres, escalate)
    info = _lib.MixedInfo()
    st = L.bola_dgesv_mixed(n, nrhs, _p(A), n, _p(b), n, _p(x), n, ctypes.byref(opts), ctypes.byref(info),
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


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
@pytest.mark.parametrize("n,nrhs", [(64, 1), (200, 3), (1000, 16), (2048, 32)])
def test_mixed_reaches_1e14_well_conditioned(kind, n, nrhs):
    A, b = make_system(n, nrhs, 1e2, seed=3)
    x, info = solve(A, b, n, nrhs, kind)
    assert info.backward_error <= 1e-14
    assert berr(A, x, b, n, nrhs) <= 1e-14
    if kind >= 2 or n <= 1000:
        # refinement (plain, or GMRES-IR for the slower bf16 factors) converged without the FP64 path
        assert info.path in (0, 1), (info.path, info.iterations)


@pytest.mark.parametrize("kappa", [1e2, 1e6, 1e10])
@pytest.mark.parametrize("kind", [0, 2])
def test_mixed_kappa_sweep_vs_oracle(oracle_lib, kappa, kind):
    n, nrhs = 1024, 4
    A, b = make_system(n, nrhs, kappa, seed=5)
    x, info = solve(A, b, n, nrhs, kind)
    assert info.backward_error <= 1e-14
    assert berr(A, x, b, n, nrhs) <= 1e-14
    A_np = A.cpu().numpy().reshape(n, n).T.copy(order="F")
    b_np = b.cpu().numpy().reshape(nrhs, n).T.copy(order="F")
    info_o, _ = oracle_lib.solve_lu(A_np, b_np)
    assert info_o == 0
    X = x.cpu().numpy().reshape(nrhs, n).T
    fwd = np.abs(X - b_np).max() / np.abs(b_np).max()
    assert fwd <= max(kappa, 10.0) * 1e-13, fwd


def test_mixed_without_fallback_reports_stall_honestly():
    n, nrhs = 512, 2
    A, b = make_system(n, nrhs, 1e10, seed=7)
    x, info = solve(A, b, n, nrhs, 0, fallback=0, max_it=10, gmres=0)
    # bf16 factors cannot refine a kappa = 1e10 system by plain IR: the call says so
    assert info.path == 0
    measured = berr(A, x, b, n, nrhs)
    assert (info.backward_error > 1e-14) == (measured > 1e-14)


@pytest.mark.parametrize("kind", [0, 2])
def test_gmres_ir_reports_truthfully_at_kappa_1e10(kind):
    """At kappa = 1e10 a TF32-accurate factor leaves ~1/3 of a geometric
    spectrum below its accuracy: GMRES(24)-IR may not converge.  Without the
    FP64 fallback the call must report exactly what it achieved."""
    n, nrhs = 1024, 4
    A, b = make_system(n, nrhs, 1e10, seed=9)
    x, info = solve(A, b, n, nrhs, kind, fallback=0)
    assert info.path in (0, 1)
    measured = berr(A, x, b, n, nrhs)
    assert abs(np.log10(max(info.backward_error, 1e-300)) - np.log10(max(measured, 1e-300))) < 0.5
    # the U-diagonal spread is a lower bound on kappa; for a bf16 factor it
    # saturates near the factor's own accuracy (a few thousand)
    assert info.condition_estimate > 1e3


def test_hopeless_refinement_goes_straight_to_fp64():
    n, nrhs = 1024, 4
    A, b = make_system(n, nrhs, 1e10, seed=9)
    x, info = solve(A, b, n, nrhs, 0, fallback=1)  # bf16 factor, kappa 1e10
    assert info.path == 2 and info.iterations == 0
    assert berr(A, x, b, n, nrhs) <= 1e-14


@pytest.mark.parametrize("kind", [0, 2])
def test_gmres_ir_handles_kappa_1e6(kind):
    n, nrhs = 1024, 4
    A, b = make_system(n, nrhs, 1e6, seed=9)
    x, info = solve(A, b, n, nrhs, kind, fallback=1)
    assert berr(A, x, b, n, nrhs) <= 1e-14
    if kind == 2:
        assert info.path in (0, 1)


@pytest.mark.parametrize("kappa", [1e6, 1e10])
@pytest.mark.parametrize("n,nrhs", [(1024, 4), (777, 3), (6500, 2)])
def test_fp64_factor_refines_ill_conditioned(kappa, n, nrhs):
    """Factor kind 3 (FP64 storage, exact-split tensor-core updates) is
    FP64-accurate: refinement reaches 1e-14 at kappa 1e10 without the FP64
    fallback, in a few sweeps.  n = 6500 takes 32-column FP64 panels first."""
    A, b = make_system(n, nrhs, kappa, seed=9)
    x, info = solve(A, b, n, nrhs, 3, fallback=0)
    assert info.path in (0, 1) and info.factor_info == 0
    assert info.backward_error <= 1e-14
    assert berr(A, x, b, n, nrhs) <= 1e-14
    assert info.iterations <= 6


@pytest.mark.parametrize("kind", [0, 2])
def test_escalation_to_fp64_accurate_factor(kind):
    """A factor that cannot refine kappa = 1e10 hands the system to the
    FP64-accurate factor (path 3) instead of the plain FP64 path."""
    n, nrhs = 1024, 4
    A, b = make_system(n, nrhs, 1e10, seed=9)
    x, info = solve(A, b, n, nrhs, kind, fallback=1, escalate=1)
    assert info.path == 3
    assert info.backward_error <= 1e-14 and berr(A, x, b, n, nrhs) <= 1e-14


def test_give_up_decides_as_the_whole_factor_would():
    """The 3xTF32 factor gives up once the U-diagonal spread reaches its limit
    or is on course for 100 times it (log-linear extrapolation from a quarter
    of the columns on); the finished factor's spread does exceed the limit,
    so the decision is the one the whole factor would give, only earlier."""
    n, nrhs = 2048, 2
    A, b = make_system(n, nrhs, 1e10, seed=11)
    _, early = solve(A, b, n, nrhs, 2, fallback=1)            # may give up
    _, full = solve(A, b, n, nrhs, 2, fallback=0, max_it=0)   # never gives up
    assert early.path == 2
    assert full.condition_estimate >= 4.5e4
    assert early.condition_estimate <= full.condition_estimate


def test_no_early_give_up_where_the_factor_refines():
    """kappa = 1e6: the spread never extrapolates past 100 times the limit, so
    the 3xTF32 factor is kept and refinement reaches the tolerance."""
    n, nrhs = 2048, 2
    A, b = make_system(n, nrhs, 1e6, seed=11)
    x, info = solve(A, b, n, nrhs, 2, fallback=1, escalate=1)
    assert info.path in (0, 1)
    assert berr(A, x, b, n, nrhs) <= 1e-14


def test_escalated_answer_equals_the_fp64_factor_alone():
    """After giving up on the 3xTF32 factor, the FP64-accurate factor starts
    from A again: the answer is the one it gives on its own."""
    n, nrhs = 1024, 3
    A, b = make_system(n, nrhs, 1e10, seed=12)
    x2, i2 = solve(A, b, n, nrhs, 2, fallback=1, escalate=1)
    x3, i3 = solve(A, b, n, nrhs, 3, fallback=1)
    assert i2.path == 3 and i3.path in (0, 1)
    assert torch.equal(x2, x3)


def test_escalation_not_taken_when_refinement_converges():
    n, nrhs = 1024, 4
    A, b = make_system(n, nrhs, 1e2, seed=9)
    x, info = solve(A, b, n, nrhs, 2, fallback=1, escalate=1)
    assert info.path in (0, 1)
    assert berr(A, x, b, n, nrhs) <= 1e-14


@pytest.mark.parametrize("n,nrhs", [(300, 3), (1001, 16), (4500, 20)])
def test_triangular_solves_with_an_odd_block_count(n, nrhs):
    """The FP32 triangular solves take 64-row blocks two at a time: an odd
    number of blocks leaves the last pair with one block; 20 right-hand sides
    take the 32-wide form.  The refinement still reaches 1e-14 by plain IR."""
    A, b = make_system(n, nrhs, 1e2, seed=13)
    x, info = solve(A, b, n, nrhs, 2)
    assert info.path == 0, (info.path, info.iterations)
    assert info.iterations <= 4
    assert berr(A, x, b, n, nrhs) <= 1e-14
