"""bola_dgemm_noalloc: the DGEMM entry point that allocates no device memory.

Who needs it: callers that must not allocate on the GPU — a real-time loop
where a cudaMalloc/pool allocation could block or fragment, an application
that owns all device memory through its own allocator, or a service running
under a fixed memory budget.  bola_dgemm borrows temporary memory for its
split-K partial sums; bola_dgemm_noalloc keeps them in a 64 MiB array built
into the library.  Each check calls both entry points through the C ABI on
the same inputs and requires bit-identical output (the tolerance of every
DGEMM test in this suite), twice in a row with fresh inputs, so nothing may
leak from one call of the shared scratch array into the next.

The file is collected last on purpose; it passes alone in a fresh process and
after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

BOLA_ERR_UNSUPPORTED = -1002


@pytest.fixture(scope="module")
def lib():
    from bola_gb300 import _lib
    return _lib.load()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _operands(ta, tb, m, n, k, seed):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    A = torch.rand((m * k,), dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    B = torch.rand((k * n,), dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    C = torch.rand((m * n,), dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    lda = max(1, m if ta == "N" else k)
    ldb = max(1, k if tb == "N" else n)
    return A, lda, B, ldb, C


def _call(lib, fn, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C):
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return getattr(lib, fn)(ta.encode(), tb.encode(), m, n, k, alpha, _ptr(A), lda, _ptr(B), ldb, beta, _ptr(C), m,
                            stream)


# split-K into the static scratch (outputs too small to fill the GPU), the
# direct path, and BOLA's unfused edge tiles
SHAPES = [
    ("N", "T", 4096, 32, 2048, -1.0, 1.0),   # Cholesky panel shape, 32 MiB of partial sums
    ("T", "N", 1001, 24, 3000, 0.5, -2.0),   # split-K plus partial 8x4 edge tiles
    ("N", "N", 300, 200, 129, 1.0, 0.0),     # split-K, beta = 0
    ("N", "N", 2048, 2048, 64, 1.0, 1.0),    # enough tiles: no scratch used
    # fewer 64x64 tiles than SMs but more than twice as many 32x32 tiles: a
    # split count taken from 32x32 tiles would not split at all here
    ("N", "N", 1024, 512, 256, 1.0, 1.0),
    ("N", "T", 512, 64, 640, 0.0, 0.5),      # alpha = 0: only the beta pass
    ("T", "T", 256, 96, 0, 2.0, -1.0),       # k = 0: only the beta pass
]


@pytest.mark.parametrize("ta,tb,m,n,k,alpha,beta", SHAPES)
def test_noalloc_matches_dgemm_twice_in_a_row(lib, ta, tb, m, n, k, alpha, beta):
    for call in range(2):
        A, lda, B, ldb, C0 = _operands(ta, tb, m, n, k, seed=1000 * call + m + n + k)
        C_ref, C_new = C0.clone(), C0.clone()
        assert _call(lib, "bola_dgemm", ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C_ref) == 0
        assert _call(lib, "bola_dgemm_noalloc", ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C_new) == 0
        torch.cuda.synchronize()
        assert torch.equal(C_ref, C_new), f"call {call}: max diff {(C_ref - C_new).abs().max().item()}"


def test_noalloc_rejects_shapes_beyond_its_scratch(lib):
    # 4096 x 32 output, K = 16384: 256 chunks x 4096 x 32 doubles = 256 MiB > 64 MiB
    ta, tb, m, n, k = "N", "T", 4096, 32, 16384
    A, lda, B, ldb, C0 = _operands(ta, tb, m, n, k, seed=7)
    C = C0.clone()
    st = _call(lib, "bola_dgemm_noalloc", ta, tb, m, n, k, 1.0, A, lda, B, ldb, 1.0, C)
    assert st == BOLA_ERR_UNSUPPORTED
    assert b"scratch" in lib.bola_last_error()
    torch.cuda.synchronize()
    assert torch.equal(C, C0)  # nothing was launched
    # the allocating entry point still handles it, and the no-alloc one keeps working afterwards
    assert _call(lib, "bola_dgemm", ta, tb, m, n, k, 1.0, A, lda, B, ldb, 1.0, C) == 0
    ta, tb, m, n, k, alpha, beta = SHAPES[0]
    A, lda, B, ldb, C0 = _operands(ta, tb, m, n, k, seed=8)
    C_ref, C_new = C0.clone(), C0.clone()
    assert _call(lib, "bola_dgemm", ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C_ref) == 0
    assert _call(lib, "bola_dgemm_noalloc", ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C_new) == 0
    torch.cuda.synchronize()
    assert torch.equal(C_ref, C_new)
