"""Small fixed workloads for profiling the library's kernels (ncu, timers).

    python profile_cases.py getrf N        # 2 x bola_dgetrf, A uniform[-1,1), seed 1
    python profile_cases.py potrf N        # 2 x bola_dpotrf('L'), A = B B^T / n + I, seed 2
    python profile_cases.py mixed N KIND   # 2 x bola_dgesv_mixed, 16 RHS, A = U[-1,1) + 4 I
    python profile_cases.py mixed N KIND E # the same on A = Q1 diag(s) Q2, kappa = 10^E, escalation on
                                    # (Q from torch's QR of seeded Gaussians: needs torch.linalg)
    python profile_cases.py batched COUNT  # 2 x bola_batch_solve, the batched workload (seed 4)

With --scopes, the library's own device timers are on during the last call
and its per-scope device time is printed after it.

Inputs are made with torch's generator on the device (no torch.linalg, so the
cases also run under profilers that cannot load its solver libraries).  Each
run prints its CUDA-event time; exit status 0 means every call succeeded.
"""
import ctypes
import sys

import torch

from bola_gb300 import _lib


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _timed(fn):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def _check(L, st, what):
    if st != 0:
        raise SystemExit(f"{what}: status {st}: {L.bola_last_error().decode()}")


def case_getrf(n):
    L = _lib.load()
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    A0 = torch.rand(n * n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    A = torch.empty_like(A0)
    ipiv = torch.empty(n, dtype=torch.int32, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        A.copy_(A0)
        ms = _timed(lambda: _check(L, L.bola_dgetrf(n, n, _p(A), n, _p(ipiv), _p(info), s), "bola_dgetrf"))
        print(f"getrf n={n} {ms:.2f} ms info={int(info)}")


def case_potrf(n):
    L = _lib.load()
    g = torch.Generator(device="cuda")
    g.manual_seed(2)
    B = torch.rand(n, n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    S0 = (B @ B.t() / n + torch.eye(n, dtype=torch.float64, device="cuda")).reshape(-1)
    S = torch.empty_like(S0)
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        S.copy_(S0)
        ms = _timed(lambda: _check(L, L.bola_dpotrf(b"L", n, _p(S), n, _p(info), s), "bola_dpotrf"))
        print(f"potrf n={n} {ms:.2f} ms info={int(info)}")


def case_mixed(n, kind, kappa_exp=None):
    L = _lib.load()
    nrhs = 16
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    if kappa_exp is None:
        A = torch.rand(n, n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
        A += 4 * torch.eye(n, dtype=torch.float64, device="cuda")
    else:
        q1, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g))
        q2, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g))
        sigma = torch.logspace(0.0, -float(kappa_exp), n, dtype=torch.float64, device="cuda")
        A = (q1 * sigma) @ q2
    A = A.t().contiguous().reshape(-1)
    b = torch.rand(n * nrhs, dtype=torch.float64, device="cuda", generator=g)
    x = torch.zeros(n * nrhs, dtype=torch.float64, device="cuda")
    opts, info = _lib.MixedOpts(kind, 30, 1e-14, 1, 1, 0 if kappa_exp is None else 1), _lib.MixedInfo()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        ms = _timed(lambda: _check(L, L.bola_dgesv_mixed(n, nrhs, _p(A), n, _p(b), n, _p(x), n, ctypes.byref(opts),
                                                         ctypes.byref(info), s), "bola_dgesv_mixed"))
        print(f"mixed n={n} kind={kind} {ms:.2f} ms path={info.path} sweeps={info.iterations} "
              f"berr={info.backward_error:.2e}")
    if info.backward_error > 1e-14:
        raise SystemExit("backward error above 1e-14")


def case_batched(count):
    from .batch import Batch, config4_batch
    ns, nrhs, kinds, fill = config4_batch(count, seed=4)
    b = Batch(ns, nrhs, kinds)
    fill(b)
    A0, B0 = b.A.clone(), b.B.clone()
    for _ in range(2):
        b.A.copy_(A0)
        b.B.copy_(B0)
        ms = _timed(lambda: b.solve())
        print(f"batched count={count} {ms:.2f} ms nonzero_info={int((b.info != 0).sum())}")
    b.close()


def _print_scopes():
    from . import api
    prof = api.profile_read()
    total = sum(v["ms"] for v in prof.values()) or 1.0
    for name, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"]):
        print(f"  {name:24s} scopes={v['calls']:6d} launches={v['launches']:6d} {v['ms']:9.3f} ms "
              f"{100 * v['ms'] / total:5.1f}%")


def main(argv):
    scopes = "--scopes" in argv
    argv = [a for a in argv if a != "--scopes"]
    if not argv:
        raise SystemExit(__doc__)
    case, args = argv[0], [int(a) for a in argv[1:]]
    fn = {"getrf": case_getrf, "potrf": case_potrf, "mixed": case_mixed, "batched": case_batched}[case]
    if scopes:
        from . import api
        fn(*args)  # warm
        api.profile_reset()
        api.profile_enable(True)
        fn(*args)
        api.profile_enable(False)
        _print_scopes()
    else:
        fn(*args)


if __name__ == "__main__":
    main(sys.argv[1:])
