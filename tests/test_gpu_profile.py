"""The device-time profiler (bola_profile_*, api.print_profile): the GPU
counterpart of BOLA's `profiling` feature (src/profiling.rs:25-115).  Checks
call counts, kernel launch counts, the 2mnk flop attribution of DGEMM (main
region and BOLA's unfused edge tiles separately), that nothing is recorded
while disabled, reset, and the report's shape."""
import numpy as np
import pytest
import torch

from bola_gb300 import api, workloads as wl

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.asfortranarray(a).ravel(order="F")).cuda()


def gemm(m, n, k, seed):
    A = dev(wl.uniform_matrix(m, k, seed=seed))
    B = dev(wl.uniform_matrix(k, n, seed=seed + 1))
    C = dev(wl.uniform_matrix(m, n, seed=seed + 2))
    api.gemm("N", "N", m, n, k, 1.0, A, m, B, k, 1.0, C, m)


@pytest.fixture
def profiler():
    api.profile_enable(False)
    api.profile_reset()
    yield
    api.profile_enable(False)
    api.profile_reset()


def test_dgemm_calls_launches_and_flops(profiler):
    api.profile_enable(True)
    for i in range(3):
        gemm(2048, 2048, 64, seed=10 + i)   # enough tiles: one launch, no split-K
    for i in range(2):
        gemm(256, 256, 4096, seed=20 + i)   # 16 tiles: split-K (partial pass + chunk-ordered fold)
    gemm(517, 383, 100, seed=30)            # partial 8x4 edge tiles: the unfused edge kernel too
    torch.cuda.synchronize()
    api.profile_enable(False)
    prof = api.profile_read()
    d = prof["dgemm"]
    assert d["calls"] == 6
    # 2048^2 x 64: one launch each; 256^2 x 4096 and the edge shape's main
    # region (64x32 tiles, fewer than the SMs, two K chunks): split-K, two
    # launches each (on GB300's 152 SMs)
    if torch.cuda.get_device_properties(0).multi_processor_count == 152:
        assert d["launches"] == 3 * 1 + 2 * 2 + 2
    else:
        assert 8 <= d["launches"] <= 9
    m8, n4 = 512, 380  # 517 -> 512 rows, 383 -> 380 columns in BOLA's full 8x4 tiles
    flops = 3 * 2.0 * 2048 * 2048 * 64 + 2 * 2.0 * 256 * 256 * 4096 + 2.0 * m8 * n4 * 100
    assert d["flops"] == pytest.approx(flops, rel=1e-12)
    e = prof["dgemm_edge"]
    assert e["calls"] == 1 and e["launches"] == 1
    ne = (517 - m8) * 383 + m8 * (383 - n4)
    assert e["flops"] == pytest.approx(2.0 * ne * 100, rel=1e-12)
    assert d["ms"] > 0 and e["ms"] > 0
    # sustained rate of the big calls is physical: below the FP64 pipe's ~1.3 TFLOP/s
    assert d["flops"] / (d["ms"] * 1e9) < 1.5


def test_disabled_records_nothing_and_reset_clears(profiler):
    gemm(256, 256, 256, seed=1)
    torch.cuda.synchronize()
    assert api.profile_read() == {}
    api.profile_enable(True)
    gemm(256, 256, 256, seed=2)
    torch.cuda.synchronize()
    assert api.profile_read()["dgemm"]["calls"] == 1
    api.profile_reset()
    assert api.profile_read() == {}


def test_factorisation_scopes(profiler):
    n = 512
    A = dev(wl.uniform_matrix(n, n, seed=3, lo=-1.0, hi=1.0))
    ipiv = torch.zeros(n, dtype=torch.int32, device="cuda")
    api.profile_enable(True)
    api.getrf(n, n, A, n, ipiv)
    torch.cuda.synchronize()
    api.profile_enable(False)
    prof = api.profile_read()
    # the blocked LU's pieces each show up with their own scope
    assert sum(v["calls"] for v in prof.values()) >= n // 32
    assert any("dgemm" in k for k in prof)
    assert all(v["ms"] >= 0 and v["launches"] >= v["calls"] > 0 for v in prof.values())


def test_report_has_bolas_columns(profiler, capsys):
    api.profile_enable(True)
    gemm(512, 512, 512, seed=4)
    torch.cuda.synchronize()
    api.profile_enable(False)
    api.print_profile()
    out = capsys.readouterr().out.splitlines()
    assert out[0].split() == ["routine", "calls", "ms", "total", "us/call", "GFLOP/s", "%", "of", "max"]
    assert out[1].startswith("dgemm")
