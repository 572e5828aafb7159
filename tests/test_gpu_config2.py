"""The plain FP64 sweep at full size (n = 4096): DGETRF with ipiv bit-exact,
DPOTRF 'L', DTRSM (L,L,N,U) with 1024 right-hand sides — each bit-identical
to the oracle, plus size-independent residual checks."""
import numpy as np
import pytest

from bola_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
N = 4096


@pytest.fixture(scope="module")
def gpu():
    from gpu_backend import GpuBackend
    return GpuBackend()


@pytest.fixture(scope="module")
def lu_pair(gpu, oracle_lib):
    A = wl.uniform_matrix(N, N, seed=1, lo=-1.0, hi=1.0)
    A1, A2 = A.copy(order="F"), A.copy(order="F")
    p1, p2 = np.zeros(N, np.int32), np.zeros(N, np.int32)
    info, margins = oracle_lib.getrf_with_margins(A1, p1)
    assert info == 0
    assert gpu.getrf(N, N, A2, N, p2) == 0
    return A, A1, p1, A2, p2, margins


def test_getrf_4096_ipiv_bit_exact(lu_pair):
    A, A1, p1, A2, p2, margins = lu_pair
    assert np.array_equal(p1, p2), f"pivots differ; smallest candidate margin {margins.min():.3e}"
    assert np.array_equal(A1, A2)


def test_getrf_4096_backward_error(lu_pair):
    A, _, _, LU, piv, _ = lu_pair
    # ||P A - L U|| / ||A|| on a 64-column sample (size-independent property)
    rng = np.random.default_rng(0)
    cols = np.sort(rng.choice(N, 64, replace=False))
    PA = A.copy()
    for i in range(N):
        p = piv[i] - 1
        if p != i:
            PA[[i, p]] = PA[[p, i]]
    L = np.tril(LU, -1) + np.eye(N)
    U = np.triu(LU)
    R = PA[:, cols] - L @ U[:, cols]
    assert np.linalg.norm(R) / np.linalg.norm(A[:, cols]) < 50 * N * np.finfo(float).eps


def test_trsm_4096x1024_bit_exact(lu_pair, gpu, oracle_lib):
    _, A1, _, _, _, _ = lu_pair
    B = wl.uniform_matrix(N, 1024, seed=1, lo=-1.0, hi=1.0, stream="trsm-rhs")
    B1, B2 = B.copy(order="F"), B.copy(order="F")
    oracle_lib.trsm("L", "L", "N", "U", N, 1024, 1.0, A1, N, B1, N)
    gpu.trsm("L", "L", "N", "U", N, 1024, 1.0, A1, N, B2, N)
    assert np.array_equal(B1, B2)


def test_potrf_4096_bit_exact(gpu, oracle_lib):
    S = wl.spd_matrix(N, seed=2)
    S1, S2 = S.copy(order="F"), S.copy(order="F")
    assert oracle_lib.potrf("L", N, S1, N) == 0
    assert gpu.potrf("L", N, S2, N) == 0
    assert np.array_equal(np.tril(S1), np.tril(S2))
    L = np.tril(S2)
    rng = np.random.default_rng(1)
    cols = np.sort(rng.choice(N, 64, replace=False))
    R = S[:, cols] - L @ L[cols, :].T
    assert np.linalg.norm(R) / np.linalg.norm(S[:, cols]) < 50 * N * np.finfo(float).eps
