"""GPU (C ABI) against the oracle on the same seeded inputs.

The FP64 routines reproduce BOLA's operation order element by element, so
the bar here is BIT-IDENTICAL output (np.array_equal), for both SIMD-width
semantics; ipiv and info must match exactly."""
import numpy as np
import pytest

import kat
from bola_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

CASES = kat.load_cases()


@pytest.fixture(scope="module")
def gpu():
    from gpu_backend import GpuBackend
    return GpuBackend()


@pytest.fixture(params=[2, 4], ids=["neon", "avx2"])
def both(request, gpu, oracle_lib):
    gpu.set_lanes(request.param)
    oracle_lib.set_lanes(request.param)
    yield gpu, oracle_lib
    gpu.set_lanes(2)
    oracle_lib.set_lanes(2)


def same(a, b):
    return np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("case", CASES, ids=[c["source"] for c in CASES])
def test_bola_known_answers_on_gpu(gpu, case):
    kat.check_case(gpu, case)


GEMM_SHAPES = [(1, 1, 1), (3, 2, 5), (8, 4, 16), (9, 5, 17), (33, 17, 65), (64, 64, 64),
               (100, 70, 129), (130, 140, 200), (257, 31, 300), (40, 300, 7)]


@pytest.mark.parametrize("ta", "NT")
@pytest.mark.parametrize("tb", "NT")
def test_gemm_bitwise(both, ta, tb):
    g, o = both
    for idx, (m, n, k) in enumerate(GEMM_SHAPES):
        for alpha, beta in [(1.0, 1.0), (-1.0, 1.0), (0.5, -2.0), (1.0, 0.0), (0.0, 3.0)]:
            A = wl.uniform_matrix(*((m, k) if ta == "N" else (k, m)), seed=idx, lo=-1, hi=1)
            B = wl.uniform_matrix(*((k, n) if tb == "N" else (n, k)), seed=idx + 50, lo=-1, hi=1)
            C = wl.uniform_matrix(m, n, seed=idx + 99, lo=-1, hi=1)
            C1, C2 = C.copy(order="F"), C.copy(order="F")
            o.gemm(ta, tb, m, n, k, alpha, A, A.shape[0], B, B.shape[0], beta, C1, m)
            g.gemm(ta, tb, m, n, k, alpha, A, A.shape[0], B, B.shape[0], beta, C2, m)
            assert same(C1, C2), (ta, tb, m, n, k, alpha, beta, np.abs(C1 - C2).max())


def test_gemm_config1_bitwise_and_within_1e12(gpu, oracle_lib):
    """DGEMM 'N','N' m=n=k=1024, A,B,C uniform [0,1) from seed 0, alpha=beta=1."""
    n = 1024
    A, B, C = wl.gemm_inputs(n, n, n, seed=0)
    C1, C2 = C.copy(order="F"), C.copy(order="F")
    oracle_lib.gemm("N", "N", n, n, n, 1.0, A, n, B, n, 1.0, C1, n)
    gpu.gemm("N", "N", n, n, n, 1.0, A, n, B, n, 1.0, C2, n)
    assert np.all(np.abs(C2 - C1) <= 1e-12 * np.abs(C1))
    assert same(C1, C2)


def test_gemm_beta_zero_clears_nan(gpu):
    m = n = k = 16
    A = wl.uniform_matrix(m, k, seed=1)
    B = wl.uniform_matrix(k, n, seed=2)
    C = np.full((m, n), np.nan, order="F")
    gpu.gemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, C, m)
    assert np.allclose(C, A @ B, rtol=1e-14)


@pytest.mark.parametrize("side,uplo,ta,diag", [(s, u, t, d) for s in "LR" for u in "LU" for t in "NT" for d in "NU"])
def test_trsm_bitwise(both, side, uplo, ta, diag):
    g, o = both
    for (m, n) in [(5, 3), (70, 9), (150, 131), (33, 200)]:
        k = m if side == "L" else n
        A = wl.uniform_matrix(k, k, seed=7, lo=-1, hi=1)
        A[np.diag_indices(k)] += np.sqrt(k) + 1.0
        B = wl.uniform_matrix(m, n, seed=8, lo=-1, hi=1)
        B1, B2 = B.copy(order="F"), B.copy(order="F")
        o.trsm(side, uplo, ta, diag, m, n, 1.5, A, k, B1, m)
        g.trsm(side, uplo, ta, diag, m, n, 1.5, A, k, B2, m)
        assert same(B1, B2), (m, n, np.abs(B1 - B2).max())


@pytest.mark.parametrize("uplo,trans", [("L", "N"), ("U", "T")])
def test_syrk_bitwise(both, uplo, trans):
    g, o = both
    for (n, k, beta) in [(3, 2, 1.0), (40, 70, 0.5), (97, 33, 0.0), (64, 130, 1.0)]:
        A = wl.uniform_matrix(*((n, k) if trans == "N" else (k, n)), seed=3, lo=-1, hi=1)
        C = wl.uniform_matrix(n, n, seed=4, lo=-1, hi=1)
        C1, C2 = C.copy(order="F"), C.copy(order="F")
        o.syrk(uplo, trans, n, k, -1.0, A, A.shape[0], beta, C1, n)
        g.syrk(uplo, trans, n, k, -1.0, A, A.shape[0], beta, C2, n)
        assert same(C1, C2), (n, k, np.abs(C1 - C2).max())


@pytest.mark.parametrize("uplo,trans", [("U", "N"), ("L", "T")])
def test_syrk_blas_definition_where_bola_misaddresses(gpu, uplo, trans):
    for (n, k) in [(20, 30), (70, 45)]:
        A = wl.uniform_matrix(*((n, k) if trans == "N" else (k, n)), seed=5, lo=-1, hi=1)
        C = np.zeros((n, n), order="F")
        gpu.syrk(uplo, trans, n, k, 1.0, A, A.shape[0], 0.0, C, n)
        opA = A if trans == "N" else A.T
        tri = np.triu if uplo == "U" else np.tril
        assert np.allclose(tri(C), tri(opA @ opA.T), rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("m,n", [(3, 3), (31, 31), (32, 32), (33, 33), (100, 100), (257, 257), (300, 200),
                                 (200, 300), (1000, 1000), (20, 90), (90, 20), (13000, 40)])
def test_getrf_bitwise(both, m, n):
    g, o = both
    A = wl.uniform_matrix(m, n, seed=m * 7 + n, lo=-1, hi=1)
    A1, A2 = A.copy(order="F"), A.copy(order="F")
    p1 = np.zeros(min(m, n), np.int32)
    p2 = np.zeros(min(m, n), np.int32)
    assert o.getrf(m, n, A1, m, p1) == 0
    assert g.getrf(m, n, A2, m, p2) == 0
    assert np.array_equal(p1, p2)
    assert same(A1, A2), np.abs(A1 - A2).max()


@pytest.mark.parametrize("m,n,pad", [(900, 600, 5), (600, 900, 3), (700, 700, 64)])
def test_getrf_lookahead_rectangular_padded(both, m, n, pad):
    """The look-ahead path (min(m, n) >= 512) on rectangular matrices whose
    leading dimension exceeds m; the padding rows must stay untouched."""
    g, o = both
    lda = m + pad
    A = np.asfortranarray(wl.uniform_matrix(lda, n, seed=m + 3 * n + pad, lo=-1, hi=1))
    A1, A2 = A.copy(order="F"), A.copy(order="F")
    p1 = np.zeros(min(m, n), np.int32)
    p2 = np.zeros(min(m, n), np.int32)
    assert o.getrf(m, n, A1, lda, p1) == 0
    assert g.getrf(m, n, A2, lda, p2) == 0
    assert np.array_equal(p1, p2)
    assert same(A1, A2)
    assert np.array_equal(A2[m:, :], A[m:, :])


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_potrf_right_looking_padded(both, uplo):
    g, o = both
    n, lda = 600, 611
    S = wl.spd_matrix(n, seed=21)
    A = np.asfortranarray(wl.uniform_matrix(lda, n, seed=22, lo=-1, hi=1))
    A[:n, :] = S
    A1, A2 = A.copy(order="F"), A.copy(order="F")
    assert o.potrf(uplo, n, A1, lda) == 0
    assert g.potrf(uplo, n, A2, lda) == 0
    assert same(A1, A2)
    assert np.array_equal(A2[n:, :], A[n:, :])


def test_getrf_ties_follow_bola_lane_order(both):
    """Integer matrices make exact pivot ties common."""
    g, o = both
    n = 96
    A = np.asfortranarray(np.floor(wl.uniform_matrix(n, n, seed=9) * 5.0) - 2.0)
    A[np.diag_indices(n)] += 0.5
    A1, A2 = A.copy(order="F"), A.copy(order="F")
    p1, p2 = np.zeros(n, np.int32), np.zeros(n, np.int32)
    r1 = o.getrf(n, n, A1, n, p1)
    r2 = g.getrf(n, n, A2, n, p2)
    assert (r1 == 0) == (r2 == 0)
    assert np.array_equal(p1, p2)
    assert same(A1, A2)


@pytest.mark.parametrize("n,col", [(100, 0), (100, 5), (100, 40), (100, 70), (100, 95), (600, 3), (600, 333),
                                   (700, 690)])
def test_getrf_singular_stops_like_bola(both, n, col):
    g, o = both
    A = wl.uniform_matrix(n, n, seed=17, lo=-1, hi=1)
    A[:, col] = 0.0
    A1, A2 = A.copy(order="F"), A.copy(order="F")
    p1, p2 = np.zeros(n, np.int32), np.zeros(n, np.int32)
    info = o.getrf(n, n, A1, n, p1)
    assert info == col + 1
    msg = g.getrf(n, n, A2, n, p2)
    local = col + 1 if n <= 32 else col % 32 + 1
    assert msg == f"Matrix is singular. The pivot in column {local} is zero."
    assert np.array_equal(p1, p2)
    assert same(A1, A2)


@pytest.mark.parametrize("n", [40, 90, 200])
def test_getrf2_recursive_bitwise(both, n):
    g, o = both
    A = wl.uniform_matrix(n, n, seed=n, lo=-1, hi=1)
    A1, A2 = A.copy(order="F"), A.copy(order="F")
    p1, p2 = np.zeros(n, np.int32), np.zeros(n, np.int32)
    assert o.getrf2(n, n, A1, n, p1) == 0
    assert g.getrf2(n, n, A2, n, p2) == 0
    assert np.array_equal(p1, p2)
    assert same(A1, A2)


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("n", [1, 3, 32, 33, 64, 100, 203, 257, 390, 545, 777])
def test_potrf_bitwise(both, uplo, n):
    g, o = both
    A = wl.spd_matrix(n, seed=n + 1)
    A1, A2 = A.copy(order="F"), A.copy(order="F")
    assert o.potrf(uplo, n, A1, n) == 0
    assert g.potrf(uplo, n, A2, n) == 0
    assert same(A1, A2), np.abs(A1 - A2).max()


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_potrf2_bitwise(both, uplo):
    g, o = both
    n = 75
    A = wl.spd_matrix(n, seed=3)
    A1, A2 = A.copy(order="F"), A.copy(order="F")
    assert o.potrf2(uplo, n, A1, n) == 0
    assert g.potrf2(uplo, n, A2, n) == 0
    assert same(A1, A2)


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("n,bad", [(100, 0), (100, 20), (100, 45), (100, 70), (100, 99), (301, 200),
                                   (600, 5), (600, 70), (600, 450), (700, 699)])
def test_potrf_not_spd(gpu, oracle_lib, uplo, n, bad):
    """BOLA stops at the failing block: later columns keep their input values."""
    A = wl.spd_matrix(n, seed=2)
    A[bad, bad] = -1000.0
    A1, A2 = A.copy(order="F"), A.copy(order="F")
    info = oracle_lib.potrf(uplo, n, A1, n)
    msg = gpu.potrf(uplo, n, A2, n)
    assert msg == f"Matrix is not positive-definite. Failure at column {(info - 1) % 32 + 1}."
    assert same(A1, A2)


def test_argument_errors(gpu):
    assert gpu.getrf(4, 4, np.zeros((4, 4), order="F"), 3, np.zeros(4, np.int32)) == \
        "Argument 4 to getrf had an illegal value of 3"
    assert gpu.potrf("l", 4, np.eye(4, order="F"), 4) == "Argument 1 to potrf had an illegal value"
    assert gpu.potrf("L", 4, np.eye(4, order="F"), 3) == "Argument 4 to potrf had an illegal value"


@pytest.mark.parametrize("k1,k2,incx", [(1, 3, 1), (2, 30, 1), (1, 60, 1), (1, 60, -1), (5, 9, -1)])
def test_laswp_bitwise(gpu, oracle_lib, k1, k2, incx):
    m, n = 80, 300
    A = wl.uniform_matrix(m, n, seed=1)
    ip = (np.floor(wl.uniform01(5, 70) * m).astype(np.int32) + 1)
    A1, A2 = A.copy(order="F"), A.copy(order="F")
    oracle_lib.laswp(n, A1, m, k1, k2, ip, incx)
    gpu.laswp(n, A2, m, k1, k2, ip, incx)
    assert np.array_equal(A1, A2)


@pytest.mark.parametrize("n", [1, 5, 7, 8, 9, 15, 16, 17, 33, 70, 1000])
def test_idamax_special_values(both, n):
    """NaN is never selected, +-inf is, zeros only on the scalar path; ties
    follow BOLA's lane order."""
    g, o = both
    rng = np.random.default_rng(n)
    cases = [np.zeros(n), np.full(n, np.nan), np.full(n, -0.0), np.full(n, 3.0)]
    x = rng.integers(-3, 4, size=n).astype(np.float64)
    x[rng.integers(0, n, size=max(1, n // 5))] = np.nan
    cases.append(x)
    y = x.copy()
    y[rng.integers(0, n)] = -np.inf
    cases.append(y)
    z = np.where(np.isnan(x), 0.0, x)
    cases.append(z)
    for v in cases:
        assert g.idamax(v) == o.idamax(v), v


def test_getrf_with_nan_and_inf_entries(both):
    g, o = both
    n = 70
    A = wl.uniform_matrix(n, n, seed=5, lo=-1, hi=1)
    A[10, 3] = np.nan
    A[50, 40] = np.inf
    A1, A2 = A.copy(order="F"), A.copy(order="F")
    p1, p2 = np.zeros(n, np.int32), np.zeros(n, np.int32)
    r1 = o.getrf(n, n, A1, n, p1)
    r2 = g.getrf(n, n, A2, n, p2)
    assert (r1 == 0) == (r2 == 0)
    assert np.array_equal(p1, p2)
    assert same(A1, A2)


def test_level1_bitwise(both):
    g, o = both
    for n in [1, 7, 8, 15, 16, 17, 100, 1001, 70000]:
        x = wl.uniform_matrix(n, 1, seed=n, lo=-1, hi=1).ravel()
        y = wl.uniform_matrix(n, 1, seed=n + 1, lo=-1, hi=1).ravel()
        assert g.idamax(x) == o.idamax(x)
        assert g.dot_product(n, x, 1, y, 1) == o.dot_product(n, x, 1, y, 1)
        y1, y2 = y.copy(), y.copy()
        o.daxpy(n, -0.7, x, 1, y1, 1)
        g.daxpy(n, -0.7, x, 1, y2, 1)
        assert same(y1, y2)
        x1, x2 = x.copy(), x.copy()
        o.scal(n, 1.0 / 3.0, x1, 1)
        g.scal(n, 1.0 / 3.0, x2, 1)
        assert same(x1, x2)
    xt = np.zeros(50)
    xt[[3, 17, 29, 45]] = -4.0
    assert g.idamax(xt) == o.idamax(xt)
    for (m, n) in [(5, 3), (37, 10), (64, 9)]:
        x = wl.uniform_matrix(m, 1, seed=m, lo=-1, hi=1).ravel()
        y = wl.uniform_matrix(n * 3, 1, seed=n, lo=-1, hi=1).ravel()
        y[0] = 0.0
        y[3] = 0.0
        A = wl.uniform_matrix(m, n, seed=m + n, lo=-1, hi=1)
        A1, A2 = A.copy(order="F"), A.copy(order="F")
        o.ger(m, n, -1.0, x, y, 3, A1, m)
        g.ger(m, n, -1.0, x, y, 3, A2, m)
        assert same(A1, A2)


def test_solve_composites_bitwise(gpu, oracle_lib):
    n, nrhs = 300, 7
    A = wl.uniform_matrix(n, n, seed=31, lo=-1, hi=1)
    B = wl.uniform_matrix(n, nrhs, seed=32, lo=-1, hi=1)
    A1, B1 = A.copy(order="F"), B.copy(order="F")
    info, piv = oracle_lib.solve_lu(A1, B1)
    A2, p2 = A.copy(order="F"), np.zeros(n, np.int32)
    assert gpu.getrf(n, n, A2, n, p2) == 0
    B2 = B.copy(order="F")
    gpu.getrs(n, nrhs, A2, n, p2, B2, n)
    assert same(B1, B2)
    S = wl.spd_matrix(n, seed=33)
    S1, C1 = S.copy(order="F"), B.copy(order="F")
    assert oracle_lib.solve_chol(S1, C1) == 0
    S2 = S.copy(order="F")
    assert gpu.potrf("L", n, S2, n) == 0
    C2 = B.copy(order="F")
    gpu.potrs("L", n, nrhs, S2, n, C2, n)
    assert same(C1, C2)


def test_repeat_runs_are_identical(gpu):
    n = 513
    A = wl.uniform_matrix(n, n, seed=77, lo=-1, hi=1)
    outs = []
    for _ in range(3):
        A2, p = A.copy(order="F"), np.zeros(n, np.int32)
        assert gpu.getrf(n, n, A2, n, p) == 0
        outs.append((A2, p))
    assert all(np.array_equal(outs[0][0], o[0]) and np.array_equal(outs[0][1], o[1]) for o in outs[1:])
