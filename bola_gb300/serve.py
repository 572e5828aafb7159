"""Solve server (bola_server_* in include/bola_gb300.h) and its request workload.

`Server` wraps the C++ server: requests are submitted from host memory and
complete asynchronously; `wait` returns the solution and the request record
(path taken, backward error, submit/admit/done times on the server's clock).

`request_pool` and `poisson_trace` build the serving workload: solve
requests arriving as a Poisson process, n log-uniform in [16, 4096], nrhs
uniform in [1, 32], 70 % general and 30 % SPD systems built from orthogonal
factors with singular values geometric from 1 to 1/kappa, kappa drawn from
{1e2, 1e6, 1e10}.  Requests draw their system from a pool generated once
(distinct seeded systems held in pinned host memory), so that generating
inputs never sits on the timed path.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib

MODES = {"mixed": 0, "fp64": 1}
PATHS = {0: "mixed-ir", 1: "gmres-ir", 2: "fp64", 3: "batched-fp64", 4: "fp64-accurate-factor"}
KAPPAS = (1e2, 1e6, 1e10)


class ServerError(RuntimeError):
    pass


class Server:
    """A running bola_server on the current CUDA device.

    mode "mixed": large requests take the mixed-precision solver (FP64
    fallback included); "fp64": the plain FP64 per-request path.  Requests
    with n <= small_n are batched (FP64); small_n=0 sends every request
    through the per-request path.
    """

    def __init__(self, slots=4, small_n=256, max_batch=256, mode="mixed", factor_kind=2,
                 hbm_budget_bytes=120 * 10**9, group_size=None, tuning=None):
        self.L = _lib.load()
        o = _lib.ServerOpts()
        o.slots, o.small_n, o.max_batch = int(slots), int(small_n), int(max_batch)
        o.mode, o.factor_kind = MODES[mode], int(factor_kind)
        if tuning is not None:  # a batch.Tuning: group sizes, panel widths, register tile
            group_size = tuning.group_size
            for i, v in enumerate(tuning.panel_width):
                o.panel_width[i] = int(v)
            o.tile_rows = int(tuning.tile_rows)
        if group_size is not None:
            for i, v in enumerate(group_size):
                o.group_size[i] = int(v)
        o.hbm_budget_bytes = int(hbm_budget_bytes)
        self.h = ctypes.c_void_p()
        st = self.L.bola_server_create(ctypes.byref(o), ctypes.byref(self.h))
        if st != 0:
            raise ServerError(f"bola_server_create: {st} {self.L.bola_last_error().decode()}")
        self._keep = {}

    @staticmethod
    def _colmajor(t):
        """Host float64 storage of matrix t in column-major order."""
        t = torch.as_tensor(t)
        if t.dim() == 1:
            t = t.reshape(-1, 1)
        if t.device.type != "cpu" or t.dtype != torch.float64:
            t = t.to("cpu", torch.float64)
        return t if t.t().is_contiguous() else t.t().contiguous().t()

    def submit(self, a, b, kind=0):
        """Queue A X = B (a: n x n, b: n x nrhs, host); returns the request id."""
        A, B = self._colmajor(a), self._colmajor(b)
        n, nrhs = A.shape[0], B.shape[1]
        if A.shape != (n, n) or B.shape[0] != n:
            raise ValueError("a must be n x n and b n x nrhs")
        rid = ctypes.c_int64()
        st = self.L.bola_server_submit(self.h, n, nrhs, int(kind), A.data_ptr(), B.data_ptr(), ctypes.byref(rid))
        if st != 0:
            raise ServerError(f"bola_server_submit: {st} {self.L.bola_last_error().decode()}")
        self._keep[rid.value] = (A, B, n, nrhs)
        return rid.value

    def submit_raw(self, n, nrhs, kind, a_ptr, b_ptr):
        """Queue a request whose column-major host buffers the caller keeps alive."""
        rid = ctypes.c_int64()
        st = self.L.bola_server_submit(self.h, n, nrhs, int(kind), a_ptr, b_ptr, ctypes.byref(rid))
        if st != 0:
            raise ServerError(f"bola_server_submit: {st} {self.L.bola_last_error().decode()}")
        self._keep[rid.value] = (None, None, n, nrhs)
        return rid.value

    def wait(self, rid, want_x=True):
        """Block until request rid is done; returns (X as n x nrhs tensor or None, record dict)."""
        _, _, n, nrhs = self._keep[rid]
        x = torch.empty(nrhs, n, dtype=torch.float64) if want_x else None
        info = _lib.RequestInfo()
        st = self.L.bola_server_wait(self.h, rid, x.data_ptr() if want_x else None, ctypes.byref(info))
        del self._keep[rid]
        rec = {"id": rid, "n": n, "nrhs": nrhs, "status": st, "path": PATHS.get(info.path, str(info.path)),
               "iterations": info.iterations, "info": info.info, "backward_error": info.backward_error,
               "factorization": "cholesky" if info.factorization == 1 else "lu",
               "t_submit": info.t_submit, "t_admit": info.t_admit, "t_done": info.t_done,
               "latency": info.t_done - info.t_submit}
        if st != 0:
            rec["error"] = self.L.bola_last_error().decode()
        return (x.t() if want_x else None), rec

    def stats(self):
        used, pend, run = ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32()
        self.L.bola_server_stats(self.h, ctypes.byref(used), ctypes.byref(pend), ctypes.byref(run))
        return {"bytes_in_use": used.value, "pending": pend.value, "running": run.value}

    def close(self):
        if self.h:
            self.L.bola_server_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _system(n, kind, kappa, gen, device):
    """A = Q1 diag(s) Q2 (kind 0) or Q diag(s) Q^T (kind 1), s geometric 1 .. 1/kappa."""
    q1, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, device=device, generator=gen))
    s = torch.logspace(0.0, -math.log10(kappa), n, dtype=torch.float64, device=device)
    if kind == 1:
        A = (q1 * s) @ q1.t()
        A = 0.5 * (A + A.t())
    else:
        q2, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, device=device, generator=gen))
        A = (q1 * s) @ q2
    return A


def request_pool(size, seed=5, nmin=16, nmax=4096, rmax=32, device="cuda"):
    """`size` distinct systems for the serving workload, in pinned host memory.

    Entry i: n log-uniform in [nmin, nmax], kind 1 (SPD) with probability 0.3,
    kappa from KAPPAS, and rmax right-hand sides b = A x_true (x_true uniform
    [-1, 1)); a request with nrhs = k uses the first k columns.  Returns a list
    of dicts with column-major host tensors "A" (n*n) and "B" (n*rmax)."""
    rng = np.random.default_rng(seed)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    pool = []
    for _ in range(size):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        kind = int(rng.random() < 0.3)
        kappa = float(KAPPAS[rng.integers(0, len(KAPPAS))])
        A = _system(n, kind, kappa, gen, device)
        xt = torch.rand(n, rmax, dtype=torch.float64, device=device, generator=gen) * 2 - 1
        B = A @ xt
        Ah = torch.empty(n * n, dtype=torch.float64, pin_memory=True)
        Bh = torch.empty(n * rmax, dtype=torch.float64, pin_memory=True)
        Ah.copy_(A.t().reshape(-1))
        Bh.copy_(B.t().reshape(-1))
        pool.append({"n": n, "kind": kind, "kappa": kappa, "A": Ah, "B": Bh})
    if str(device).startswith("cuda"):
        torch.cuda.synchronize(device)
    return pool


def poisson_trace(rate, count, pool_size, seed=5, rmax=32):
    """Arrival times (s, from 0) of `count` requests at `rate` per second, with
    each request's pool entry and nrhs (uniform in [1, rmax])."""
    rng = np.random.default_rng([seed, int(rate * 1000)])
    t = np.cumsum(rng.exponential(1.0 / rate, size=count))
    t -= t[0]
    entry = rng.integers(0, pool_size, size=count)
    nrhs = rng.integers(1, rmax + 1, size=count)
    return t, entry, nrhs


def run_trace(server, pool, trace, want_x=False):
    """Submit the requests of `trace` at their arrival times, then collect
    every record.  Latency = done - submit on the server's clock."""
    import time
    t, entry, nrhs = trace
    ids = []
    t0 = time.perf_counter()
    for k in range(len(t)):
        delay = t[k] - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        p = pool[int(entry[k])]
        ids.append(server.submit_raw(p["n"], int(nrhs[k]), p["kind"], p["A"].data_ptr(), p["B"].data_ptr()))
    recs, xs = [], []
    for rid in ids:
        x, rec = server.wait(rid, want_x=want_x)
        recs.append(rec)
        xs.append(x)
    return recs, xs


def summarize(recs):
    """p50 / p99 latency (ms), solves/s over the trace and backward-error stats."""
    lat = np.array([r["latency"] for r in recs]) * 1e3
    t_first = min(r["t_submit"] for r in recs)
    t_last = max(r["t_done"] for r in recs)
    berr = np.array([r["backward_error"] for r in recs])
    paths, facts = {}, {}
    for r in recs:
        paths[r["path"]] = paths.get(r["path"], 0) + 1
        f = r.get("factorization", "lu")
        facts[f] = facts.get(f, 0) + 1
    return {"requests": len(recs), "solves_per_s": len(recs) / (t_last - t_first),
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "max_backward_error": float(berr.max()), "within_1e-14": int((berr <= 1e-14).sum()),
            "errors": int(sum(1 for r in recs if r["status"] != 0)), "paths": paths, "factorizations": facts}


def knee(by_rate):
    """The first offered rate whose served rate falls below 90 % of it (the
    server saturates there), with the p99 latency on either side; None if it
    kept up at every rate."""
    rates = sorted(by_rate, key=float)
    for i, r in enumerate(rates):
        if by_rate[r]["solves_per_s"] < 0.9 * float(r):
            prev = rates[i - 1] if i > 0 else None
            return {"saturates_at_rate": float(r), "served_solves_per_s": by_rate[r]["solves_per_s"],
                    "p99_ms": by_rate[r]["p99_ms"], "p99_ms_below": by_rate[prev]["p99_ms"] if prev else None}
    return None
