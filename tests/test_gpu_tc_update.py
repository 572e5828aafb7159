"""tcgen05 rank-64 update W -= A B^T against a torch FP32 reference of the
same operation (bf16, tf32 and 3xTF32 operand forms).

Shapes cover both kernels: a leading dimension that is not a multiple of 4
takes the one-tile-per-CTA kernel, the others the pipelined kernel, with
partial row and column tiles, padding rows below m (which must stay
untouched, also when m is not a multiple of 4: the pipelined kernel's tile
store stops at m & ~3 and the last rows go by plain stores) and, at 4096,
runs of several tiles per CTA."""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def tf32_split(x):
    """x ~ hi + lo with hi, lo exactly representable in tf32 (10-bit mantissa)."""
    xi = x.view(torch.int32)
    hi = ((xi + 0x1000) & ~0x1FFF).view(torch.float32)   # round to nearest tf32
    lo_full = x - hi
    lo = ((lo_full.view(torch.int32) + 0x1000) & ~0x1FFF).view(torch.float32)
    return hi.contiguous(), lo.contiguous()


@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("m,n,ldw", [(128, 128, 128), (300, 200, 301), (1000, 77, 1000), (500, 300, 516),
                                   (501, 300, 516), (1023, 130, 1028), (3, 64, 8),
                                   (2048, 2048, 2048), (4096, 4096, 4096)])
def test_tc_update_matches_fp32_reference(kind, m, n, ldw):
    from bola_gb300 import _lib
    L = _lib.load()
    g = torch.Generator(device="cuda")
    g.manual_seed(m * 7 + n + kind)
    A = torch.rand(m, 64, device="cuda", generator=g) * 2 - 1
    B = torch.rand(n, 64, device="cuda", generator=g) * 2 - 1
    W = torch.rand(n, ldw, device="cuda", generator=g)  # column-major m x n with ld ldw: row j of this = column j
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    if kind == 0:
        Ab, Bb = A.to(torch.bfloat16).contiguous(), B.to(torch.bfloat16).contiguous()
        ref_prod = Ab.float() @ Bb.float().T
        args = (_p(Ab), _p(Bb), _p(Ab), _p(Bb))
        tol = 1e-4
    elif kind == 1:
        Ah, _ = tf32_split(A)
        Bh, _ = tf32_split(B)
        ref_prod = Ah.double() @ Bh.double().T
        args = (_p(Ah), _p(Bh), _p(Ah), _p(Bh))
        tol = 1e-4
    else:
        Ah, Al = tf32_split(A)
        Bh, Bl = tf32_split(B)
        ref_prod = A.double() @ B.double().T
        args = (_p(Ah), _p(Bh), _p(Al), _p(Bl))
        tol = 2e-5
    W0 = W.clone()
    st = L.bola_sgemm_tc_update(kind, m, n, *args, _p(W), ldw, _p(err),
                                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, L.bola_last_error()
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    got = W[:, :m].T.double()           # m x n
    ref = W0[:, :m].T.double() - ref_prod
    assert torch.allclose(got, ref, atol=tol, rtol=0), (got - ref).abs().max().item()
    # the padding rows beyond m stay untouched
    if ldw > m:
        assert torch.equal(W[:, m:], W0[:, m:])
