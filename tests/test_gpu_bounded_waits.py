"""Failure detection without a GPU fault: waits that nothing can satisfy give
up after their poll limit, report it through the error word, and leave the
context usable (a DGEMM right after still matches the oracle)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_expired_waits_report_and_context_survives(oracle_lib):
    from bola_gb300 import _lib, api
    L = _lib.load()
    fe = torch.zeros(2, dtype=torch.int32, device="cuda")
    st = L.bola_selftest_bounded_waits(ctypes.c_void_p(fe.data_ptr()), 2000,
                                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    assert int(fe[0]) == 3  # the mbarrier wait and the flag wait both gave up
    # the context is still good
    rng = np.random.default_rng(3)
    a, b, c = (rng.random((64, 64)) for _ in range(3))
    c1 = np.asfortranarray(c.copy())
    oracle_lib.gemm("N", "N", 64, 64, 64, 1.0, np.asfortranarray(a), 64, np.asfortranarray(b), 64, 1.0, c1, 64)
    ta = torch.from_numpy(np.asfortranarray(a).ravel(order="F")).cuda()
    tb = torch.from_numpy(np.asfortranarray(b).ravel(order="F")).cuda()
    tc = torch.from_numpy(np.asfortranarray(c).ravel(order="F")).cuda()
    api.gemm("N", "N", 64, 64, 64, 1.0, ta, 64, tb, 64, 1.0, tc, 64)
    assert np.array_equal(tc.cpu().numpy().reshape(64, 64, order="F"), c1)


@pytest.mark.parametrize("csize,nbytes", [(2, 2176), (16, 2176), (16, 528)])
def test_cluster_exchange_probe(csize, nbytes):
    """The exchange-latency probe completes (no wait expires) and gives a
    plausible time per round: above the ~0.1 us of a shared-memory round
    trip, far below a millisecond."""
    from bola_gb300 import _lib
    L = _lib.load()
    us = ctypes.c_double(0.0)
    st = L.bola_measure_cluster_exchange(csize, nbytes, ctypes.byref(us))
    assert st == 0, L.bola_last_error()
    assert 0.05 < us.value < 100.0, us.value


def test_cluster_exchange_probe_rejects_bad_arguments():
    from bola_gb300 import _lib
    L = _lib.load()
    us = ctypes.c_double(0.0)
    assert L.bola_measure_cluster_exchange(17, 512, ctypes.byref(us)) == -1
    assert L.bola_measure_cluster_exchange(4, 100, ctypes.byref(us)) == -2


def test_fp64_throughput_probes():
    """DFMA and DMMA probes both run and give plausible FP64 rates (GB300:
    about 1.2 TFLOP/s through DFMA)."""
    from bola_gb300 import _lib
    L = _lib.load()
    v = ctypes.c_double(0.0)
    assert L.bola_measure_fp64_peak(ctypes.byref(v)) == 0, L.bola_last_error()
    assert 100.0 < v.value < 20000.0, v.value
    assert L.bola_measure_dmma_peak(ctypes.byref(v)) == 0, L.bola_last_error()
    assert 10.0 < v.value < 20000.0, v.value
