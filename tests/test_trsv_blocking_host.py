"""The block recurrence of the FP32 dataflow triangular solves (`trsv_words`
in bola_gb300/csrc/ir.cu), restated in numpy and checked against a direct
triangular solve: 64-row blocks taken in solve order by clusters of 8, each
block coupled to its last six predecessors through C_d = Dinv_b T[b, b-+d],
older blocks folded in through T.  The kernel forms the same sums in FP32;
here they run in FP64, so the recurrence itself is checked to FP64 accuracy
(partial last block, fewer blocks than couplings, several clusters, the
split of predecessors between pushes (d <= rank) and published words)."""
import numpy as np
import pytest
import scipy.linalg

TB, TCL, TNP = 64, 8, 6


def blocked_solve(T, y, lower):
    n = T.shape[0]
    nb = -(-n // TB)
    rows = [slice(b * TB, min(n, (b + 1) * TB)) for b in range(nb)]
    unit = lower

    def dinv(b):
        D = T[rows[b], rows[b]].copy()
        if unit:
            np.fill_diagonal(D, 1.0)
        return np.linalg.inv(np.tril(D) if lower else np.triu(D))

    x = np.zeros_like(y)
    for t in range(nb):
        b = t if lower else nb - 1 - t
        rank = t % TCL
        kc = min(t, TNP)
        acc = y[rows[b]].copy()
        for s in range(t - kc):  # folds: blocks before the coupled predecessors
            k = s if lower else nb - 1 - s
            acc -= T[rows[b], rows[k]] @ x[rows[k]]
        Di = dinv(b)
        cv = Di @ acc
        # coupled predecessors: from words (d > rank) first, then pushes, furthest first
        order = [d for d in range(kc, 0, -1) if d > rank] + [d for d in range(kc, 0, -1) if d <= rank]
        for d in order:
            p = b - d if lower else b + d
            C = Di @ T[rows[b], rows[p]]
            cv -= C @ x[rows[p]]
        x[rows[b]] = cv
    return x


@pytest.mark.parametrize("n", [1, 63, 64, 300, 449, 1001, 1100])
@pytest.mark.parametrize("lower", [True, False], ids=["unit-lower", "upper"])
def test_block_recurrence_matches_direct_solve(n, lower):
    rng = np.random.default_rng(n)
    nrhs = 3 if n < 500 else 16
    A = rng.uniform(-1, 1, (n, n)) / np.sqrt(n)
    if lower:
        T = np.tril(A, -1) + np.eye(n)
    else:
        T = np.triu(A, 1) + np.diag(rng.uniform(1, 2, n) * rng.choice([-1, 1], n))
    y = rng.uniform(-1, 1, (n, nrhs))
    x = blocked_solve(T, y, lower)
    ref = scipy.linalg.solve_triangular(T, y, lower=lower, unit_diagonal=lower)
    assert np.allclose(x, ref, rtol=1e-10, atol=1e-10 * np.abs(ref).max())
