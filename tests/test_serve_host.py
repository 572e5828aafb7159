"""Host-side pieces of the solve server: the arrival trace, the latency
summary and the ABI's behaviour without a device."""
import numpy as np
import pytest


def test_poisson_trace_is_seeded_and_has_the_rate():
    from bola_gb300.serve import poisson_trace
    t1, e1, r1 = poisson_trace(200.0, 4000, pool_size=32, seed=5)
    t2, e2, r2 = poisson_trace(200.0, 4000, pool_size=32, seed=5)
    assert np.array_equal(t1, t2) and np.array_equal(e1, e2) and np.array_equal(r1, r2)
    assert t1[0] == 0.0 and np.all(np.diff(t1) >= 0)
    rate = (len(t1) - 1) / t1[-1]
    assert abs(rate - 200.0) / 200.0 < 0.06
    assert e1.min() >= 0 and e1.max() < 32
    assert r1.min() == 1 and r1.max() == 32
    # a different rate gives a different trace
    t3, _, _ = poisson_trace(100.0, 4000, pool_size=32, seed=5)
    assert not np.array_equal(t1, t3)


def test_summary_percentiles():
    from bola_gb300.serve import summarize
    recs = [{"latency": (k + 1) * 1e-3, "t_submit": 0.01 * k, "t_done": 0.01 * k + (k + 1) * 1e-3,
             "backward_error": 1e-16 if k else 2e-14, "status": 0, "path": "mixed-ir" if k % 2 else "batched-fp64"}
            for k in range(100)]
    s = summarize(recs)
    assert s["requests"] == 100
    assert s["p50_ms"] == pytest.approx(50.5)
    assert s["p99_ms"] == pytest.approx(99.01)
    assert s["within_1e-14"] == 99 and s["errors"] == 0
    assert s["paths"] == {"batched-fp64": 50, "mixed-ir": 50}
    assert s["solves_per_s"] == pytest.approx(100 / (0.99 + 0.1))


def test_server_without_device_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from bola_gb300.serve import Server, ServerError
    with pytest.raises(ServerError, match="bola_server_create"):
        Server(slots=1)
