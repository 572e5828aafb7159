"""Solve server: every request of a mixed trace reaches backward error <= 1e-14;
each result is bit-identical alone and in the mix; the plain FP64 path is
bit-identical to the oracle's BOLA composite solve; admission never holds
more device bytes than the budget; argument errors are reported."""
import threading

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pool():
    from bola_gb300.serve import request_pool
    return request_pool(10, seed=51, nmin=16, nmax=600, rmax=8)


def _trace(pool, count, seed):
    rng = np.random.default_rng(seed)
    return (np.zeros(count), rng.integers(0, len(pool), size=count), rng.integers(1, 9, size=count))


def test_mixed_trace_accuracy_and_alone_equals_mix(pool):
    from bola_gb300.serve import Server, run_trace
    tr = _trace(pool, 40, seed=52)
    with Server(slots=3, small_n=128, max_batch=64) as srv:
        recs, xs = run_trace(srv, pool, tr, want_x=True)
    assert all(r["status"] == 0 for r in recs), [r for r in recs if r["status"] != 0][:2]
    assert max(r["backward_error"] for r in recs) <= 1e-14
    paths = {r["path"] for r in recs}
    assert "batched-fp64" in paths and paths & {"mixed-ir", "gmres-ir", "fp64"}
    # the same requests one at a time: identical bits
    with Server(slots=1, small_n=128, max_batch=64) as srv:
        for k in range(0, 40, 3):
            p = pool[int(tr[1][k])]
            rid = srv.submit_raw(p["n"], int(tr[2][k]), p["kind"], p["A"].data_ptr(), p["B"].data_ptr())
            x, rec = srv.wait(rid, want_x=True)
            assert rec["status"] == 0 and rec["path"] == recs[k]["path"]
            assert torch.equal(x, xs[k]), (k, p["n"], rec["path"])


def test_fp64_path_matches_oracle(pool, oracle_lib):
    from bola_gb300.serve import Server
    with Server(slots=2, small_n=0, mode="fp64") as srv:
        picks = [i for i, p in enumerate(pool) if p["n"] <= 400][:4]
        ids = []
        for i in picks:
            p = pool[i]
            ids.append(srv.submit_raw(p["n"], 3, p["kind"], p["A"].data_ptr(), p["B"].data_ptr()))
        for i, rid in zip(picks, ids):
            p, n = pool[i], pool[i]["n"]
            x, rec = srv.wait(rid, want_x=True)
            assert rec["status"] == 0 and rec["path"] == "fp64" and rec["backward_error"] <= 1e-14
            A = p["A"].numpy().reshape(n, n).T.copy(order="F")
            B = p["B"].numpy()[: 3 * n].reshape(3, n).T.copy(order="F")
            if p["kind"] == 1:
                assert oracle_lib.solve_chol(A, B) == 0
            else:
                assert oracle_lib.solve_lu(A, B)[0] == 0
            assert np.array_equal(x.numpy(), B), (n, p["kind"])


def test_admission_stays_within_budget(pool):
    from bola_gb300.serve import Server, ServerError
    big = max(pool, key=lambda p: p["n"])
    n = big["n"]
    # room for about two large requests at a time
    budget = 2 * (20 * n * n + 424 * n * 8 + 4096 * 2 + 16 * 64 * n)
    with Server(slots=4, small_n=0, hbm_budget_bytes=budget) as srv:
        seen, stop = [], threading.Event()

        def watch():
            while not stop.is_set():
                seen.append(srv.stats()["bytes_in_use"])

        th = threading.Thread(target=watch)
        th.start()
        ids = [srv.submit_raw(n, 8, big["kind"], big["A"].data_ptr(), big["B"].data_ptr()) for _ in range(8)]
        recs = [srv.wait(i, want_x=False)[1] for i in ids]
        stop.set()
        th.join()
        assert all(r["status"] == 0 for r in recs)
        assert max(seen) <= budget and max(seen) > 0
        # the budget admits two at a time: when a request is admitted, at most
        # one earlier admitted request is still running
        spans = sorted((r["t_admit"], r["t_done"]) for r in recs)
        for k in range(len(spans)):
            running = sum(1 for j in range(k) if spans[j][1] > spans[k][0] + 1e-9)
            assert running <= 1, (k, spans)
        with pytest.raises(ServerError, match="-5"):
            srv.submit_raw(4096, 32, 0, big["A"].data_ptr(), big["B"].data_ptr())


def test_argument_errors(pool):
    from bola_gb300.serve import Server, ServerError
    p = pool[0]
    with Server(slots=1) as srv:
        for args, code in (((0, 1, 0), "-2"), ((8193, 1, 0), "-2"), ((p["n"], 0, 0), "-3"),
                           ((p["n"], 33, 0), "-3"), ((p["n"], 1, 2), "-4")):
            with pytest.raises(ServerError, match=code):
                srv.submit_raw(*args, p["A"].data_ptr(), p["B"].data_ptr())
        st = srv.L.bola_server_wait(srv.h, 12345, None, None)
        assert st == -2
