"""Batched small solves in one persistent launch: accuracy against numpy's
FP64 solve, bit-equality of each system alone and in the mix, CUDA-graph
replay, and failures (singular / not SPD) confined to their own system."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _batch(count, seed, **kw):
    from bola_gb300.batch import Batch, config4_batch
    ns, nrhs, kinds, fill = config4_batch(count, seed=seed, **kw)
    b = Batch(ns, nrhs, kinds)
    fill(b)
    return b


def _snapshot(b):
    return b.A.clone(), b.B.clone()


def test_batch_matches_fp64_solve():
    b = _batch(300, seed=11, nmin=1, nmax=256)
    A0, B0 = _snapshot(b)
    b.solve()
    torch.cuda.synchronize()
    assert int(b.info.abs().sum()) == 0
    for i in range(b.count):
        n, r = int(b.ns[i]), int(b.nrhs[i])
        A = A0[int(b.a_off[i]):int(b.a_off[i + 1])].view(n, n).t().cpu().numpy()
        B = B0[int(b.b_off[i]):int(b.b_off[i + 1])].view(r, n).t().cpu().numpy()
        X = b.b_view(i).cpu().numpy()
        R = B - A @ X
        berr = np.abs(R).max(0) / (np.abs(A).sum(1).max() * np.abs(X).max(0) + np.abs(B).max(0))
        assert berr.max() < 1e-15 * max(n, 8), (i, n, berr.max())
        assert np.allclose(X, np.linalg.solve(A, B), rtol=1e-10, atol=1e-12)


def test_alone_equals_in_the_mix():
    from bola_gb300.batch import Batch
    big = _batch(400, seed=12)
    A0, B0 = _snapshot(big)
    big.solve()
    torch.cuda.synchronize()
    pick = [0, 1, 7, 33, 120, 399]
    alone = Batch(big.ns[pick], big.nrhs[pick], big.kinds[pick])
    for j, i in enumerate(pick):
        alone.a_view(j).copy_(A0[int(big.a_off[i]):int(big.a_off[i + 1])].view(int(big.ns[i]), -1).t())
        alone.b_view(j).copy_(B0[int(big.b_off[i]):int(big.b_off[i + 1])].view(int(big.nrhs[i]), -1).t())
    alone.solve()
    torch.cuda.synchronize()
    for j, i in enumerate(pick):
        assert torch.equal(alone.b_view(j), big.b_view(i)), i
        assert torch.equal(alone.a_view(j), big.a_view(i)), i


def test_graph_replay_is_identical():
    b = _batch(200, seed=13)
    A0, B0 = _snapshot(b)
    b.solve(graph=True)
    torch.cuda.synchronize()
    X1 = b.B.clone()
    b.A.copy_(A0)
    b.B.copy_(B0)
    b.solve(graph=True)
    torch.cuda.synchronize()
    assert torch.equal(X1, b.B)


def test_failures_stay_in_their_system():
    b = _batch(64, seed=14)
    A0, B0 = _snapshot(b)
    b.solve()
    torch.cuda.synchronize()
    X_ok = b.B.clone()
    # system 10 (LU): zero column 3; system 11 (Cholesky): negative diagonal
    b.A.copy_(A0)
    b.B.copy_(B0)
    b.a_view(10)[:, 3] = 0.0
    b.a_view(11)[5, 5] = -1e6
    b.solve()
    torch.cuda.synchronize()
    info = b.info.cpu().numpy()
    assert info[10] > 0 and info[11] == 6
    others = [i for i in range(b.count) if i not in (10, 11)]
    assert (info[others] == 0).all()
    for i in others:
        assert torch.equal(b.b_view(i), X_ok[int(b.b_off[i]):int(b.b_off[i + 1])].view(int(b.nrhs[i]), -1).t())


def test_every_tuning_choice_is_bit_identical():
    """Group size, panel width and register tile change the schedule, never
    an element's operation order: every choice gives the same bits."""
    from bola_gb300.batch import Tuning
    b = _batch(160, seed=21, nmin=1, nmax=256)
    A0, B0 = _snapshot(b)
    b.solve()
    torch.cuda.synchronize()
    ref_A, ref_B = b.A.clone(), b.B.clone()
    for g, pw, tr in [(32, 12, 4), (64, 16, 2), (128, 8, 2), (256, 12, 4), (32, 16, 2)]:
        b.A.copy_(A0)
        b.B.copy_(B0)
        b.replan(Tuning([g] * 8, [pw] * 8, tr))
        b.solve()
        torch.cuda.synchronize()
        assert torch.equal(b.A, ref_A) and torch.equal(b.B, ref_B), (g, pw, tr)


def test_autotuned_plan_is_persisted_bit_identical_and_no_slower(tmp_path):
    from bola_gb300.batch import Batch, Tuning, autotune, time_solve
    b = _batch(2000, seed=4)
    A0, B0 = _snapshot(b)
    b.solve()
    torch.cuda.synchronize()
    ref_B = b.B.clone()
    b.A.copy_(A0)
    b.B.copy_(B0)
    path = tmp_path / "batched_tuning.json"
    tuned, trials = autotune(b, reps=2, path=path)
    loaded, _ = Tuning.load(path)  # what a later process loads at plan creation
    assert loaded.as_dict() == tuned.as_dict()
    fresh = Batch(b.ns, b.nrhs, b.kinds, tuning=loaded)
    fresh.A.copy_(A0)
    fresh.B.copy_(B0)
    fresh.solve()
    torch.cuda.synchronize()
    assert torch.equal(fresh.B, ref_B)
    b.replan(None)  # the built-in defaults
    t_default = time_solve(b, A0, B0, 5, graph=False)  # (minimum over the repetitions)
    t_tuned = time_solve(fresh, A0, B0, 5, graph=False)
    # the tuned table is the measured best of a set that contains the defaults
    assert t_tuned <= 1.10 * t_default, (t_tuned, t_default, tuned.as_dict())
    fresh.close()
    b.close()
