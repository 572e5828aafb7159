"""FP64-accurate rank-64 update on the bf16 tensor cores (exact slicing):
exact on integer data; otherwise within 2^-44 * 64 * max|a_i.| * max|b_j.|
of the FP64 product (the slicing works relative to each row's scale);
ragged tile edges, an odd leading dimension (no L2 prefetch of W) and, at
4096 x 2000, several tiles per CTA included."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _run(A, B, W):
    from bola_gb300 import _lib
    L = _lib.load()
    m, n = W.shape
    a = torch.from_numpy(np.ascontiguousarray(A)).cuda()  # m x 64, K-major rows
    b = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    w = torch.from_numpy(np.asfortranarray(W).T.copy().reshape(-1)).cuda()  # column-major m x n
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = L.bola_dgemm_oz_update(m, n, a.data_ptr(), b.data_ptr(), w.data_ptr(), m, err.data_ptr(),
                                torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert st == 0, L.bola_last_error()
    assert int(err) == 0
    return w.cpu().numpy().reshape(n, m).T


@pytest.mark.parametrize("m,n", [(300, 200), (128, 64), (1000, 513), (1001, 700), (4096, 2000)])
def test_integer_data_is_exact(m, n):
    rng = np.random.default_rng(m + n)
    A = rng.integers(-100, 101, size=(m, 64)).astype(np.float64)
    B = rng.integers(-100, 101, size=(n, 64)).astype(np.float64)
    W = rng.integers(-10**6, 10**6, size=(m, n)).astype(np.float64)
    ref = (W.astype(np.int64) - A.astype(np.int64) @ B.astype(np.int64).T).astype(np.float64)
    assert np.array_equal(_run(A, B, W), ref)


@pytest.mark.parametrize("m,n", [(700, 300), (2048, 1024)])
def test_scaled_rows_within_row_scale_bound(m, n):
    rng = np.random.default_rng(7)
    A = rng.standard_normal((m, 64)) * 10.0 ** rng.uniform(-3, 3, size=(m, 1))
    B = rng.standard_normal((n, 64)) * 10.0 ** rng.uniform(-3, 3, size=(n, 1))
    A[:, 5] *= 1e-6  # small entries inside a row
    W = rng.standard_normal((m, n))
    got = _run(A, B, W)
    ref = W - A @ B.T
    scale = np.outer(np.abs(A).max(1), np.abs(B).max(1))
    bound = 2.0 ** -44 * 64 * scale + 4 * np.finfo(float).eps * np.abs(ref)
    assert np.all(np.abs(got - ref) <= bound)
    # and far tighter than FP32 arithmetic would be
    assert np.median(np.abs(got - ref) / scale) < 2.0 ** -46
