"""The oracle (CPU restatement of BOLA) pinned against BOLA's own known-answer
tests, then against the mathematical definitions at sizes the known answers
do not reach (multi-block paths, recursion, both SIMD-width semantics)."""
import numpy as np
import pytest

import kat
from bola_gb300 import workloads as wl

CASES = kat.load_cases()


@pytest.fixture(params=[2, 4], ids=["neon", "avx2"])
def orc(request, oracle_lib):
    oracle_lib.set_lanes(request.param)
    yield oracle_lib
    oracle_lib.set_lanes(2)


@pytest.mark.parametrize("case", CASES, ids=[c["source"] for c in CASES])
def test_bola_known_answers(orc, case):
    kat.check_case(orc, case)


def test_gemm_all_transposes_vs_numpy(orc):
    rng = np.random.default_rng(5)
    for ta in "NT":
        for tb in "NT":
            for (m, n, k) in [(1, 1, 1), (7, 5, 3), (33, 17, 65), (130, 140, 129)]:
                A = np.asfortranarray(rng.uniform(-1, 1, (m, k) if ta == "N" else (k, m)))
                B = np.asfortranarray(rng.uniform(-1, 1, (k, n) if tb == "N" else (n, k)))
                C = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
                ref = 0.5 * (A if ta == "N" else A.T) @ (B if tb == "N" else B.T) - 2.0 * C
                orc.gemm(ta, tb, m, n, k, 0.5, A, A.shape[0], B, B.shape[0], -2.0, C, m)
                assert np.allclose(C, ref, rtol=1e-12, atol=1e-12)


def test_gemm_thread_count_does_not_change_bits(oracle_lib):
    rng = np.random.default_rng(1)
    A = np.asfortranarray(rng.uniform(0, 1, (300, 200)))
    B = np.asfortranarray(rng.uniform(0, 1, (200, 260)))
    C0 = np.asfortranarray(rng.uniform(0, 1, (300, 260)))
    outs = []
    for t in (1, 3, 0):
        oracle_lib.set_threads(t)
        C = C0.copy(order="F")
        oracle_lib.gemm("N", "N", 300, 260, 200, 1.0, A, 300, B, 200, 1.0, C, 300)
        outs.append(C)
    oracle_lib.set_threads(0)
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


@pytest.mark.parametrize("side,uplo,ta,diag", [(s, u, t, d) for s in "LR" for u in "LU" for t in "NT" for d in "NU"])
def test_trsm_all_variants_vs_numpy(orc, side, uplo, ta, diag):
    rng = np.random.default_rng(7)
    for (m, n) in [(5, 3), (70, 9), (150, 131)]:
        k = m if side == "L" else n
        A = rng.uniform(-1, 1, (k, k)) + 4 * k * np.eye(k) * 0 + np.diag(rng.uniform(1, 2, k)) * k ** 0.5
        A = np.asfortranarray(A)
        B = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
        T = np.tril(A) if uplo == "L" else np.triu(A)
        if diag == "U":
            np.fill_diagonal(T, 1.0)
        opT = T if ta == "N" else T.T
        X = B.copy(order="F")
        orc.trsm(side, uplo, ta, diag, m, n, 1.5, A, k, X, m)
        ref = np.linalg.solve(opT, 1.5 * B) if side == "L" else np.linalg.solve(opT.T, 1.5 * B.T).T
        assert np.allclose(X, ref, rtol=1e-9, atol=1e-9), (m, n)


@pytest.mark.parametrize("uplo,trans", [("L", "N"), ("U", "T")])
def test_syrk_correct_combinations_vs_numpy(orc, uplo, trans):
    rng = np.random.default_rng(3)
    for (n, k) in [(3, 2), (40, 70), (97, 33)]:
        A = np.asfortranarray(rng.uniform(-1, 1, (n, k) if trans == "N" else (k, n)))
        C = np.asfortranarray(rng.uniform(-1, 1, (n, n)))
        opA = A if trans == "N" else A.T
        ref = -1.0 * opA @ opA.T + 0.5 * C
        out = C.copy(order="F")
        orc.syrk(uplo, trans, n, k, -1.0, A, A.shape[0], 0.5, out, n)
        tri = np.tril if uplo == "L" else np.triu
        assert np.allclose(tri(out), tri(ref), rtol=1e-12, atol=1e-12)
        other = np.triu(out, 1) if uplo == "L" else np.tril(out, -1)
        assert np.array_equal(other, (np.triu(C, 1) if uplo == "L" else np.tril(C, -1)))


@pytest.mark.parametrize("uplo,trans", [("U", "N"), ("L", "T")])
def test_syrk_bola_addressing_quirk(orc, uplo, trans):
    """BOLA addresses the diagonal block of A wrongly for (U,N) and (L,T)
    (src/syrk.rs:80 and :139): exact for n,k <= 32, wrong beyond."""
    rng = np.random.default_rng(4)
    for (n, k, exact) in [(20, 30, True), (40, 70, False)]:
        A = np.asfortranarray(rng.uniform(-1, 1, (n, k) if trans == "N" else (k, n)))
        C = np.zeros((n, n), order="F")
        opA = A if trans == "N" else A.T
        orc.syrk(uplo, trans, n, k, 1.0, A, A.shape[0], 0.0, C, n)
        tri = np.tril if uplo == "L" else np.triu
        ok = np.allclose(tri(C), tri(opA @ opA.T), rtol=1e-12, atol=1e-12)
        assert ok == exact


def test_getrf_residual_and_pivots(orc):
    for n in (3, 31, 32, 33, 100, 257):
        A0 = wl.uniform_matrix(n, n, seed=11, lo=-1.0, hi=1.0)
        A = A0.copy(order="F")
        ipiv = np.zeros(n, dtype=np.int32)
        assert orc.getrf(n, n, A, n, ipiv) == 0
        L = np.tril(A, -1) + np.eye(n)
        U = np.triu(A)
        PA = A0.copy()
        for i in range(n):
            p = ipiv[i] - 1
            PA[[i, p]] = PA[[p, i]]
        assert np.linalg.norm(PA - L @ U) <= 1e-13 * n * np.linalg.norm(A0)
        # partial pivoting: every multiplier is bounded by one
        assert np.max(np.abs(np.tril(A, -1))) <= 1.0


def test_getrf2_recursive_path_matches_definition(orc):
    """getrf2 on a matrix wider and taller than 32 takes the recursive branch
    (src/getrf2.rs:54-103), which getrf itself never reaches."""
    n = 90
    A0 = wl.uniform_matrix(n, n, seed=12, lo=-1.0, hi=1.0)
    A = A0.copy(order="F")
    ipiv = np.zeros(n, dtype=np.int32)
    assert orc.getrf2(n, n, A, n, ipiv) == 0
    L = np.tril(A, -1) + np.eye(n)
    U = np.triu(A)
    PA = A0.copy()
    for i in range(n):
        p = ipiv[i] - 1
        PA[[i, p]] = PA[[p, i]]
    assert np.linalg.norm(PA - L @ U) <= 1e-13 * n * np.linalg.norm(A0)


def test_getrf_singular_and_bad_lda(orc):
    n = 70
    A = wl.uniform_matrix(n, n, seed=13, lo=-1.0, hi=1.0)
    A[:, 40] = 0.0
    ipiv = np.zeros(n, dtype=np.int32)
    assert orc.getrf(n, n, A, n, ipiv) == 41
    assert orc.getrf(4, 4, np.zeros((4, 4), order="F"), 3, np.zeros(4, np.int32)) == -4


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_potrf_vs_numpy(orc, uplo):
    for n in (3, 32, 33, 100):
        A0 = wl.spd_matrix(n, seed=21)
        A = A0.copy(order="F")
        assert orc.potrf(uplo, n, A, n) == 0
        L = np.linalg.cholesky(A0)
        got = np.tril(A) if uplo == "L" else np.triu(A).T
        assert np.allclose(got, L, rtol=1e-11, atol=1e-11)


def test_potrf_errors(orc):
    A = wl.spd_matrix(50, seed=2)
    A[45, 45] = -100.0
    assert orc.potrf("L", 50, A.copy(order="F"), 50) == 46
    assert orc.potrf("l", 50, A.copy(order="F"), 50) == -1
    assert orc.potrf("L", 50, A.copy(order="F"), 40) == -4


def test_laswp_negative_increment(orc):
    a = np.asfortranarray(np.arange(12, dtype=np.float64).reshape(4, 3, order="F"))
    ref = a.copy(order="F")
    ipiv = np.array([3, 4, 3], dtype=np.int32)
    orc.laswp(3, a, 4, 1, 3, ipiv, -1)
    for i, p in [(3, 3), (2, 4), (1, 3)]:  # backwards over k2..k1
        ref[[i - 1, p - 1]] = ref[[p - 1, i - 1]]
    assert np.array_equal(a, ref)


def test_idamax_tie_rule(orc):
    # equal magnitudes: with SIMD lanes BOLA does not always return the first
    x = np.zeros(40)
    x[[5, 21]] = 3.0
    got = orc.idamax(x)
    assert got in (5, 21)
    lanes = orc.get_lanes()
    # lane of index 5 vs 21 under the 4-accumulator interleave
    def prio(i):
        chunk = 4 * lanes
        r = i % chunk
        return (r % lanes, r // lanes, i // chunk)
    assert got == min([5, 21], key=prio)


def test_solve_composites(oracle_lib):
    n, nrhs = 120, 5
    A0 = wl.uniform_matrix(n, n, seed=31, lo=-1.0, hi=1.0)
    X0 = wl.uniform_matrix(n, nrhs, seed=32, lo=-1.0, hi=1.0)
    B = np.asfortranarray(A0 @ X0)
    A = A0.copy(order="F")
    info, _ = oracle_lib.solve_lu(A, B)
    assert info == 0 and np.allclose(B, X0, atol=1e-10)
    S = wl.spd_matrix(n, seed=33)
    B = np.asfortranarray(S @ X0)
    assert oracle_lib.solve_chol(S.copy(order="F"), B) == 0
    assert np.allclose(B, X0, atol=1e-10)
