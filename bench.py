#!/usr/bin/env python
"""Dense LU solve throughput on one GB300 (the BOLA getrf + trsm solve path).

Workload: n = 8192, 16 right-hand sides, A = Q1 diag(sigma) Q2 with Q1, Q2
from the Householder QR of Gaussian matrices (seed 3), sigma geometric from 1
to 1/kappa; the timed steps rotate over kappa = 1e2, 1e6, 1e10; b = A x_true,
x_true uniform [-1, 1).  One step = one complete solve of A x = b (factor +
solve), whose normwise backward error is checked to be <= 1e-14.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours       the C-ABI library on the GPU: `value` is the mixed-precision solve
           (bola_dgesv_mixed: 3xTF32 tensor-core LU + FP64 refinement; a system
           that factor cannot refine is solved again with the FP64-accurate
           factor: FP64 panels, exact bf16 slicing of the trailing update on the
           tensor cores; plain FP64 as the last resort) with inputs in HBM;
           `plain_fp64` is the BOLA-exact FP64 path (bola_dgetrf + bola_dgetrs)
           on the same systems; `e2e` copies A and b from pinned host memory
           every step and reads x back (the next system's copy on a copy
           stream during the current solve, into a second device buffer).
           The library's device profiler (CUDA events on the launching
           stream, in a second pass over the timed steps) gives the
           per-kernel roofline numbers and the launch count.
reference  BOLA's CPU algorithm (the C restatement under oracle/, all host
           threads) on the same inputs.
Under torchrun each rank solves its own systems (replicas, no collective);
value = all ranks' solves / max rank time.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402
import torch  # noqa: E402

METRIC = "solves/s and p99 latency, mixed-prec IR vs plain FP64 at ≤1e-14 backward error"
KAPPAS = (1e2, 1e6, 1e10)
BERR_TARGET = 1e-14


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--nrhs", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-systems", type=int, default=20000)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-plain-configs", action="store_true")
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[25.0, 50.0, 100.0, 200.0, 400.0, 800.0, 1600.0])
    ap.add_argument("--serve-requests", type=int, default=300)
    ap.add_argument("--serve-pool", type=int, default=128)
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-forward-error", action="store_true")
    return ap.parse_args()


# ---------------------------------------------------------------- inputs ----

def make_systems(n, nrhs, device):
    """Config-3 systems, built with torch on `device` (input preparation only)."""
    from bola_gb300 import workloads as wl
    g1 = torch.from_numpy(wl.gaussian_matrix(n, n, seed=3, stream="q1")).to(device)
    g2 = torch.from_numpy(wl.gaussian_matrix(n, n, seed=3, stream="q2")).to(device)
    q1, _ = torch.linalg.qr(g1)
    del g1
    q2, _ = torch.linalg.qr(g2)
    del g2
    x_true = torch.from_numpy(wl.uniform_matrix(n, nrhs, seed=3, lo=-1.0, hi=1.0, stream="x")).to(device)
    systems = []
    for kappa in KAPPAS:
        sigma = torch.logspace(0.0, -np.log10(kappa), n, dtype=torch.float64, device=device)
        A = (q1 * sigma) @ q2
        b = A @ x_true
        # column-major flat storage, as the C ABI takes it
        systems.append({"kappa": kappa, "A": A.t().contiguous().reshape(-1), "b": b.t().contiguous().reshape(-1),
                        "x_true": x_true})
    del q1, q2
    torch.cuda.synchronize(device)
    return systems


def backward_error(A_flat, x_flat, b_flat, n, nrhs):
    """max over right-hand sides of ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf)."""
    A = A_flat.reshape(n, n).t()
    X = x_flat.reshape(nrhs, n).t()
    B = b_flat.reshape(nrhs, n).t()
    R = B - A @ X
    a_inf = A.abs().sum(dim=1).max()
    num = R.abs().max(dim=0).values
    den = a_inf * X.abs().max(dim=0).values + B.abs().max(dim=0).values
    return float((num / den).max())


# ---------------------------------------------------------------- clocks ----

class ClockSampler:
    """nvidia-smi SM clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path:
            return None
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows), "reasons": reasons}


# ---------------------------------------------------------------- ours ----

class Solver:
    """Plain FP64 solve through the C ABI: getrf (BOLA's blocked LU, exact)
    then getrs (laswp + two trsm), on one stream."""

    def __init__(self, n, nrhs, device):
        from bola_gb300 import _lib
        self.L = _lib.load()
        self.n, self.nrhs = n, nrhs
        self.work = torch.empty(n * n, dtype=torch.float64, device=device)
        self.x = torch.empty(n * nrhs, dtype=torch.float64, device=device)
        self.bdev = torch.empty(n * nrhs, dtype=torch.float64, device=device)
        self.ipiv = torch.empty(n, dtype=torch.int32, device=device)
        self.info = torch.zeros(1, dtype=torch.int32, device=device)
        self.stream = torch.cuda.current_stream(device)
        self.sp = ctypes.c_void_p(self.stream.cuda_stream)

    def _p(self, t):
        return ctypes.c_void_p(t.data_ptr())

    def solve_device(self, A, b):
        """A, b resident on the device; result in self.x (device)."""
        self.work.copy_(A)
        self.x.copy_(b)
        self._factor_solve()

    def solve_host(self, A_host, b_host, x_host):
        """Pinned host A, b in; pinned host x out."""
        self.work.copy_(A_host, non_blocking=True)
        self.x.copy_(b_host, non_blocking=True)
        self._factor_solve()
        x_host.copy_(self.x, non_blocking=True)

    def solve_mixed(self, A, b, kind=2):
        """bola_dgesv_mixed; returns the bola_mixed_info of the call."""
        from bola_gb300 import _lib
        opts = _lib.MixedOpts(kind, 30, BERR_TARGET, 1, 1, 1)
        info = _lib.MixedInfo()
        st = self.L.bola_dgesv_mixed(self.n, self.nrhs, self._p(A), self.n, self._p(b), self.n, self._p(self.x),
                                     self.n, ctypes.byref(opts), ctypes.byref(info), self.sp)
        if st != 0:
            raise RuntimeError(f"bola_dgesv_mixed status {st}: {self.L.bola_last_error().decode()}")
        return info

    def _factor_solve(self):
        n, L = self.n, self.L
        st = L.bola_dgetrf(n, n, self._p(self.work), n, self._p(self.ipiv), self._p(self.info), self.sp)
        if st != 0:
            raise RuntimeError(f"bola_dgetrf status {st}: {L.bola_last_error().decode()}")
        st = L.bola_dgetrs(n, self.nrhs, self._p(self.work), n, self._p(self.ipiv), self._p(self.x), n, self.sp)
        if st != 0:
            raise RuntimeError(f"bola_dgetrs status {st}: {L.bola_last_error().decode()}")


def max_over_ranks(values, world, device):
    """Each timing (ms) as the maximum over the ranks of a replica run (the
    slowest rank sets the job's time); unchanged for one rank."""
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(v) for v in t]


def job_rate(world, steps, total_ms):
    """Whole-job solves/s: every rank solves `steps` systems in at most total_ms."""
    return world * steps / (total_ms / 1e3)


def time_steps(fn, steps, stream):
    """CUDA-event time of each step on `stream`; synchronised on both sides."""
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    evs[0].record(stream)
    for k in range(steps):
        fn(k)
        evs[k + 1].record(stream)
    torch.cuda.synchronize()
    per = [evs[k].elapsed_time(evs[k + 1]) for k in range(steps)]
    total = evs[0].elapsed_time(evs[-1])
    return total, per


def run_ours(args, rank, world, device):
    from bola_gb300 import api
    torch.cuda.set_device(device)
    n, nrhs = args.n, args.nrhs
    systems = make_systems(n, nrhs, device)
    solver = Solver(n, nrhs, device)
    stream = solver.stream
    peak_fp64 = api.measure_fp64_peak()
    infos = []

    def step(k):
        s = systems[k % len(systems)]
        infos.append((s["kappa"], solver.solve_mixed(s["A"], s["b"])))

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    # every system once, outside the timed region: the answer must meet the
    # target, and its forward error against the oracle's FP64 solve (BOLA's
    # getrf + laswp + two trsm, on the host cores) is reported
    berr, paths, fwd = {}, {}, {}
    for s in systems:
        info = solver.solve_mixed(s["A"], s["b"])
        torch.cuda.synchronize()
        key = f"{s['kappa']:.0e}"
        berr[key] = backward_error(s["A"], solver.x, s["b"], n, nrhs)
        if not args.no_forward_error:
            _, x_or = cpu_solve_once(*host_system(s, n, nrhs))
            x = solver.x.cpu().numpy().reshape(nrhs, n).T
            x_true = s["x_true"].cpu().numpy()
            fwd[key] = {"vs_oracle": float(np.abs(x - x_or).max() / np.abs(x_or).max()),
                        "oracle_vs_x_true": float(np.abs(x_or - x_true).max() / np.abs(x_true).max()),
                        "kappa_u": s["kappa"] * 2.0 ** -53}
        paths[key] = {"path": ["mixed-IR", "mixed-GMRES-IR", "fp64-fallback", "fp64-accurate-factor-IR"][info.path],
                      "iterations": info.iterations, "gmres_iterations": info.gmres_iterations,
                      "reported_backward_error": info.backward_error}

    if world > 1:
        torch.distributed.barrier()
    infos.clear()
    with ClockSampler(device.index if device.index is not None else 0) as clk:
        total_ms, per = time_steps(step, args.steps, stream)
    # the per-kernel table (and the roofline) from a second pass over the same
    # steps with the library's device timers on: their events between kernels
    # cost time, so the timed pass above runs without them
    infos_timed = list(infos)
    api.profile_reset()
    api.profile_enable(True)
    time_steps(step, args.steps, stream)
    api.profile_enable(False)
    prof = api.profile_read()
    infos[:] = infos_timed
    if world > 1:
        torch.distributed.barrier()

    # the plain FP64 path on the same systems (BOLA-exact getrf + getrs)
    plain_steps = max(1, min(3, args.steps))

    def step_plain(k):
        s = systems[k % len(systems)]
        solver.solve_device(s["A"], s["b"])

    step_plain(0)
    plain_total, plain_per = time_steps(step_plain, plain_steps, stream)

    # end to end: pinned host buffers, every step's copies inside the timed
    # region.  Two device buffers: the next system's host->device copy runs
    # on a copy stream while the current system is solved (a solve reads its
    # A until it returns, so a buffer is refilled only after its solve).
    host = [{"A": s["A"].cpu().pin_memory(), "b": s["b"].cpu().pin_memory()} for s in systems]
    x_host = torch.empty(n * nrhs, dtype=torch.float64).pin_memory()
    cstream = torch.cuda.Stream(device)
    bufs = [(torch.empty_like(solver.work), torch.empty_like(solver.bdev)) for _ in range(2)]
    copied = [torch.cuda.Event() for _ in range(2)]
    freed = [torch.cuda.Event() for _ in range(2)]

    def enqueue_copy(k):
        h = host[k % len(host)]
        A_d, b_d = bufs[k % 2]
        with torch.cuda.stream(cstream):
            cstream.wait_event(freed[k % 2])
            A_d.copy_(h["A"], non_blocking=True)
            b_d.copy_(h["b"], non_blocking=True)
            copied[k % 2].record(cstream)

    def make_step(nsteps):
        def step_e2e(k):
            if k == 0:
                cstream.wait_stream(stream)  # the first copy starts inside the timed region
                enqueue_copy(0)
            if k + 1 < nsteps:
                enqueue_copy(k + 1)  # overlaps this solve
            stream.wait_event(copied[k % 2])
            A_d, b_d = bufs[k % 2]
            solver.solve_mixed(A_d, b_d)
            x_host.copy_(solver.x, non_blocking=True)
            freed[k % 2].record(stream)
        return step_e2e

    # the same warm-up as the device-resident steps: every host buffer and
    # both device buffers have been through a copy before the timed steps
    warm = make_step(args.warmup)
    for k in range(args.warmup):
        warm(k)
    e2e_total, e2e_per = time_steps(make_step(args.steps), args.steps, stream)

    total_ms, e2e_total, plain_total = max_over_ranks([total_ms, e2e_total, plain_total], world, device)
    if rank != 0:
        return None

    # roofline of the dominant kernel (largest share of device time)
    dom_name, dom = max(prof.items(), key=lambda kv: kv[1]["ms"])
    prof_total = sum(v["ms"] for v in prof.values())
    # exchange rounds of the cluster panels, measured on this device (floors
    # of the latency-bound panels' rooflines)
    xcache = {}

    def exchange_us(c, nbytes):
        c2 = 1 << max(0, (int(c) - 1).bit_length())  # the next power of two at or above c
        if (c2, nbytes) not in xcache:
            xcache[(c2, nbytes)] = api.measure_cluster_exchange(max(2, c2), nbytes)
        return xcache[(c2, nbytes)]

    roof = roofline_for(dom_name, dom, peak_fp64, n=n, exchange_us=exchange_us)
    roof["timing"] = ("CUDA events around each launch on its stream, in a second pass over the same steps "
                      "(the timed pass runs without them)")
    kernels = {k: {"scopes": v["calls"], "launches": v["launches"], "ms": round(v["ms"], 3),
                   "share": round(v["ms"] / prof_total, 4),
                   "tflops": round(v["flops"] / max(v["ms"], 1e-9) / 1e9, 4) if v["flops"] else None,
                   "gbs": round(v["bytes"] / max(v["ms"], 1e-9) / 1e6, 1) if v["bytes"] else None}
               for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"])}
    launches = int(sum(v["launches"] for v in prof.values()))

    value = job_rate(world, args.steps, total_ms)
    plain_value = job_rate(world, plain_steps, plain_total)
    out = {
        "metric": METRIC, "value": round(value, 4), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: A = Q1 diag(sigma) Q2, Q from Householder QR of Gaussian matrices (seed 3), sigma "
                "geometric 1..1/kappa, kappa in {1e2,1e6,1e10} rotating per step; b = A x_true, x_true U[-1,1)",
        "config": {"workload": f"dense LU solve n={n} nrhs={nrhs} to backward error <= {BERR_TARGET:g}",
                   "path": "mixed: 3xTF32 tcgen05 LU (FP32 storage, per-block-column scaling) + FP64 iterative "
                           "refinement; escalation to the FP64-accurate factor (exact-split bf16 tcgen05 "
                           "updates) when refinement cannot converge; plain FP64 last",
                   "replicas": "one independent solve stream per GPU (no collective)",
                   "l2": "inputs larger than L2 (512 MiB matrix per step)"},
        "latency_ms": {"p50": round(statistics.median(per), 3),
                       "p99": round(float(np.percentile(per, 99)), 3),
                       "median_by_kappa": {f"{systems[q]['kappa']:.0e}": round(statistics.median(per[q::len(systems)]), 3)
                                           for q in range(min(len(systems), len(per)))}},
        "plain_fp64": {"value": round(plain_value, 4), "unit": "solves/s", "steps": plain_steps,
                       "ms_per_step": round(plain_total / plain_steps, 3),
                       "path": "BOLA-exact bola_dgetrf + bola_dgetrs (FP64, NB=32)"},
        "speedup_vs_plain_fp64": round(value / plain_value, 3),
        "backward_error": berr,
        "backward_error_ok": all(v <= BERR_TARGET for v in berr.values()),
        "forward_error": fwd,
        "refinement": paths,
        "e2e": {"value": round(job_rate(world, args.steps, e2e_total), 4), "unit": "solves/s",
                "h2d_bytes_per_step": 8 * (n * n + n * nrhs), "d2h_bytes_per_step": 8 * n * nrhs,
                "overlap": "the next system's host-to-device copy runs on a copy stream during the current solve",
                "ms_per_step": round(e2e_total / args.steps, 3),
                "latency_ms": {"p50": round(statistics.median(e2e_per), 3),
                               "p99": round(float(np.percentile(e2e_per, 99)), 3)},
                "per_step_ms": [round(x, 2) for x in e2e_per]},
        "roofline": roof,
        "kernels": kernels,
        "gpu_launches": launches,
    }
    clocks = clk.summary()
    if clocks is not None:
        out["clocks"] = clocks
    if not args.no_plain_configs:
        out["factor_kinds"] = run_factor_kinds(systems, n, nrhs, device)
        out["plain_configs"] = run_plain_configs(device, peak_fp64)
    if not args.no_batched:
        out["batched"] = run_batched(args, device, peak_fp64)
    if not args.no_serve:
        out["serve"] = run_serve(args, device)
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(systems[0], n, nrhs, budget_s=12.0)
    return out


def run_batched(args, device, peak_fp64):
    """20,000 independent systems (n uniform in [8, 256], half LU on
    diagonally dominant, half Cholesky on SPD matrices, nrhs uniform in
    [1, 8], seed 4) solved in one persistent launch replayed from a CUDA
    graph; group size and panel width autotuned per size bucket, and the
    register tile per plan, in this run."""
    from bola_gb300.batch import Batch, autotune, config4_batch, time_solve
    count = args.batch_systems
    ns, nrhs, kinds, fill = config4_batch(count, seed=4, device=device)
    b = Batch(ns, nrhs, kinds, device=device)
    fill(b)
    A0, B0 = b.A.clone(), b.B.clone()
    tuning, trials = autotune(b)
    b.replan(tuning)
    b.solve(graph=True)
    torch.cuda.synchronize()
    ok_info = int((b.info != 0).sum()) == 0
    # accuracy on a sample of systems
    rng = np.random.default_rng(4)
    worst = 0.0
    for i in rng.choice(count, size=min(200, count), replace=False):
        n, r = int(ns[i]), int(nrhs[i])
        A = A0[int(b.a_off[i]):int(b.a_off[i + 1])].view(n, n).t()
        B = B0[int(b.b_off[i]):int(b.b_off[i + 1])].view(r, n).t()
        X = b.b_view(int(i))
        R = B - A @ X
        den = A.abs().sum(1).max() * X.abs().max(0).values + B.abs().max(0).values
        worst = max(worst, float((R.abs().max(0).values / den).max()))
    steps = max(3, args.steps)
    times = []
    for _ in range(steps):
        times.append(time_solve(b, A0, B0, 1, graph=True))
    n64 = ns.astype(np.float64)
    flops = float(np.sum(np.where(kinds == 1, n64 ** 3 / 3, 2 * n64 ** 3 / 3) + 2 * n64 ** 2 * nrhs))
    ms = statistics.median(times)
    b.close()
    return {"workload": f"{count} systems, n U[8,256], nrhs U[1,8], half LU / half Cholesky, seed 4",
            "systems_per_s": round(count / (ms / 1e3), 1), "ms_per_batch": round(ms, 3),
            "ms_min": round(min(times), 3), "steps": steps, "launches_per_batch": 1, "graph": True,
            "gflops": round(flops / (ms / 1e3) / 1e9, 1),
            "fp64_peak_frac": round(flops / (ms / 1e3) / 1e9 / peak_fp64, 4) if peak_fp64 else None,
            "tuning": tuning.as_dict(),
            "autotune_ms": {str(k): {str(g): round(t, 3) for g, t in v.items()} for k, v in trials.items()},
            "info_all_zero": ok_info, "max_backward_error_sample": worst}


def run_plain_configs(device, peak_fp64):
    """The BOLA-exact FP64 drop-ins at their published sizes: DGEMM NN 1024
    (alpha = beta = 1, A, B, C U[0,1)), DGETRF 4096 (U[-1,1)), DPOTRF 'L' 4096
    (B B^T / n + I), DTRSM L,L,N,U 4096 x 1024 with the unit-lower factor of
    that getrf.  Median of 5 calls after 2 warm-up calls, each timed alone with
    CUDA events; a 256 MiB buffer is rewritten between calls (L2 flushed)."""
    from bola_gb300 import _lib
    L = _lib.load()
    st = torch.cuda.current_stream()
    sp = ctypes.c_void_p(st.cuda_stream)

    def P(t):
        return ctypes.c_void_p(t.data_ptr())

    def ok(status, what):
        if status != 0:
            raise RuntimeError(f"{what}: status {status}: {L.bola_last_error().decode()}")

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)

    def timed(fn, prep):
        ts = []
        for r in range(7):
            prep()
            flush.fill_(r)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            torch.cuda.synchronize()
            if r >= 2:
                ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    def entry(ms, flops):
        gf = flops / (ms / 1e3) / 1e9
        return {"ms": round(ms, 3), "gflops": round(gf, 1),
                "fp64_peak_frac": round(gf / peak_fp64, 4) if peak_fp64 else None}

    g = torch.Generator(device=device)
    out = {"peak_fp64_gflops": round(peak_fp64, 1) if peak_fp64 else None}
    n = 1024
    g.manual_seed(0)
    A = torch.rand(n * n, dtype=torch.float64, device=device, generator=g)
    B = torch.rand(n * n, dtype=torch.float64, device=device, generator=g)
    C0 = torch.rand(n * n, dtype=torch.float64, device=device, generator=g)
    C = torch.empty_like(C0)
    ms = timed(lambda: ok(L.bola_dgemm(b"N", b"N", n, n, n, 1.0, P(A), n, P(B), n, 1.0, P(C), n, sp), "dgemm"),
               lambda: C.copy_(C0))
    out["dgemm_nn_1024"] = entry(ms, 2.0 * n ** 3)
    n = 4096
    A = torch.rand(n * n, dtype=torch.float64, device=device, generator=g)
    B = torch.rand(n * n, dtype=torch.float64, device=device, generator=g)
    C0 = torch.rand(n * n, dtype=torch.float64, device=device, generator=g)
    C = torch.empty_like(C0)
    ms = timed(lambda: ok(L.bola_dgemm(b"N", b"N", n, n, n, 1.0, P(A), n, P(B), n, 1.0, P(C), n, sp), "dgemm"),
               lambda: C.copy_(C0))
    out["dgemm_nn_4096"] = entry(ms, 2.0 * n ** 3)
    del B, C0, C
    g.manual_seed(1)
    A0 = torch.rand(n * n, dtype=torch.float64, device=device, generator=g) * 2 - 1
    ipiv = torch.empty(n, dtype=torch.int32, device=device)
    info = torch.zeros(1, dtype=torch.int32, device=device)
    ms = timed(lambda: ok(L.bola_dgetrf(n, n, P(A), n, P(ipiv), P(info), sp), "dgetrf"), lambda: A.copy_(A0))
    out["dgetrf_4096"] = entry(ms, 2.0 * n ** 3 / 3 - n ** 2 / 2 + 5.0 * n / 6)
    out["dgetrf_4096"]["info"] = int(info)
    LU = A.clone()
    g.manual_seed(11)
    X0 = torch.rand(n * 1024, dtype=torch.float64, device=device, generator=g) * 2 - 1
    X = torch.empty_like(X0)
    ms = timed(lambda: ok(L.bola_dtrsm(b"L", b"L", b"N", b"U", n, 1024, 1.0, P(LU), n, P(X), n, sp), "dtrsm"),
               lambda: X.copy_(X0))
    out["dtrsm_llnu_4096x1024"] = entry(ms, float(n) * n * 1024 - n * 1024)
    del LU, X0, X
    g.manual_seed(2)
    Bm = torch.rand(n, n, dtype=torch.float64, device=device, generator=g) * 2 - 1
    S0 = (Bm @ Bm.t() / n + torch.eye(n, dtype=torch.float64, device=device)).reshape(-1)
    del Bm
    ms = timed(lambda: ok(L.bola_dpotrf(b"L", n, P(A), n, P(info), sp), "dpotrf"), lambda: A.copy_(S0))
    out["dpotrf_l_4096"] = entry(ms, n ** 3 / 3 + n ** 2 / 2 + n / 6)
    out["dpotrf_l_4096"]["info"] = int(info)
    return out


def run_factor_kinds(systems, n, nrhs, device):
    """Config 3 per factor precision: each kind (0 bf16, 1 tf32, 2 3xTF32 with
    FP32 storage, 3 FP64-accurate) on each kappa, escalation and fallback on,
    median of 2 timed solves after one warm-up."""
    from bola_gb300 import _lib
    L = _lib.load()
    st = torch.cuda.current_stream()
    sp = ctypes.c_void_p(st.cuda_stream)
    x = torch.zeros(n * nrhs, dtype=torch.float64, device=device)
    out = {}
    names = {0: "bf16", 1: "tf32", 2: "3xtf32", 3: "fp64-accurate"}
    for kind in (0, 1, 2, 3):
        row = {}
        for sysd in systems:
            opts, info = _lib.MixedOpts(kind, 30, BERR_TARGET, 1, 1, 1), _lib.MixedInfo()
            ts = []
            for r in range(3):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                status = L.bola_dgesv_mixed(n, nrhs, ctypes.c_void_p(sysd["A"].data_ptr()), n,
                                            ctypes.c_void_p(sysd["b"].data_ptr()), n, ctypes.c_void_p(x.data_ptr()),
                                            n, ctypes.byref(opts), ctypes.byref(info), sp)
                e1.record(st)
                torch.cuda.synchronize()
                if status != 0:
                    raise RuntimeError(f"bola_dgesv_mixed: {L.bola_last_error().decode()}")
                if r >= 1:
                    ts.append(e0.elapsed_time(e1))
            row[f"{sysd['kappa']:.0e}"] = {
                "ms": round(statistics.median(ts), 3),
                "path": ["IR", "GMRES-IR", "fp64-fallback", "escalated-to-fp64-accurate"][info.path],
                "iterations": info.iterations, "gmres_iterations": info.gmres_iterations,
                "backward_error": info.backward_error, "condition_estimate": info.condition_estimate}
        out[names[kind]] = row
    return out


def run_serve(args, device):
    """The serving loop: Poisson arrivals (seed 5) at swept rates of requests
    with n log-uniform in [16, 4096], nrhs U[1, 32], 70 % LU / 30 % SPD,
    kappa in {1e2, 1e6, 1e10}; mixed server (tensor-core LU, or Cholesky for
    the SPD requests, + FP64 refinement, small requests batched) against the
    plain FP64 per-request server; inputs from pinned host memory, results
    copied back.  The sweep runs until each server saturates (its knee)."""
    from bola_gb300.serve import Server, knee, poisson_trace, request_pool, run_trace, summarize
    pool = request_pool(args.serve_pool, seed=5, device=device)
    out = {"workload": f"{args.serve_requests} requests per rate from a pool of {args.serve_pool} seeded systems "
                       f"(mean n {np.mean([p['n'] for p in pool]):.0f}), 4 slots, admission budget 120 GB",
           "rates": list(args.serve_rates), "mixed": {}, "fp64": {}}
    for mode, small in (("mixed", 256), ("fp64", 0)):
        with Server(slots=4, small_n=small, mode=mode) as srv:
            # warm-up: one request of every pool entry
            for k in range(len(pool)):
                p = pool[k]
                srv.wait(srv.submit_raw(p["n"], 4, p["kind"], p["A"].data_ptr(), p["B"].data_ptr()), want_x=False)
            for rate in args.serve_rates:
                tr = poisson_trace(rate, args.serve_requests, len(pool), seed=5)
                recs, _ = run_trace(srv, pool, tr)
                out[mode][str(rate)] = summarize(recs)
        out[mode + "_knee"] = knee(out[mode])
    return out


# DRAM bytes (read + write) per algorithmic byte, from the ncu captures
# summarised under profiles/ (n=4096 cases): the tournament panel 0.82 MB read
# for a 2816 x 64 FP32 panel whose algorithmic read + write is 1.44 MB;
# tc_update 49.4 MB for a 3392 x 3328 step with 90.3 MB algorithmic (writes
# still in L2); oz_update 129.4 MB for 180.6 MB.
TRAFFIC_PER_ALGORITHMIC_BYTE = {"tpanel": 0.57, "tc_update": 0.55, "oz_update": 0.72}


# The tournament panels of the mixed LU as slu.cu schedules them: (mp, jb, C,
# R) per panel of an n x n factorisation, 64 columns, CTAs of up to 256
# threads x 2 rows.  The same kernel selects the FP64-accurate factor's
# pivots (tselect64) on the same schedule.
def panel_schedule(n):
    out, j = [], 0
    while j < n:
        mp = n - j
        jb = min(64, mp)
        C = min(16, max(1, -(-mp // 256)))
        out.append((mp, jb, C, -(-mp // C)))
        j += jb
    return out


TSLOT_BYTES = 16 + 64 * 4   # a tournament nominee pushed between CTAs


def panel_floor(n, exchange_us):
    """Lower bound (us) of one factorisation's tournament panels and their
    unit count: per group of 8 columns, the larger of one exchange round of 8
    nominees at the panel's cluster size (measured) and the group's FP32 work
    per CTA (rank-8 update of R rows over the remaining columns) at 128 FMA
    per clock per SM, 2.07 GHz."""
    fma_sm = 128 * 2.07e9
    total, units = 0.0, 0
    sched = panel_schedule(n)
    for mp, jb, C, R in sched:
        x = exchange_us(C, 8 * TSLOT_BYTES)
        for g0 in range(0, jb, 8):
            total += max(x, 1e6 * R * 8 * (64 - g0) / fma_sm)
            units += 1
    return total, units, len(sched)


def roofline_for(name, v, peak_fp64_gflops, n=None, exchange_us=None):
    """The dominant kernel's achieved rate against its bounding peak.
    FP64 kernels: DFMA peak measured in this run.  Tensor-core update: HBM
    (it reads and writes the FP32 trailing matrix once per step).  Cluster
    panels: latency-bound; time per column (or pivot group) against a floor
    from measured exchange rounds and arithmetic rates, HBM fraction kept as
    a secondary field.  Others: HBM bytes of their algorithmic traffic."""
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    secs = v["ms"] * 1e-3
    if name in ("dgemm", "mixed_residual", "dgemm_edge"):
        ach = v["flops"] / secs / 1e12
        pk = peak_fp64_gflops / 1e3
        return {"kernel": name, "bound": "fp64", "achieved": round(ach, 4), "peak": round(pk, 4), "unit": "TFLOP/s",
                "frac": round(ach / pk, 4), "traffic": None,
                "peak_source": "FP64 DFMA throughput measured in this run (bola_measure_fp64_peak)"}
    ach = v["bytes"] / secs / 1e9
    out = {"kernel": name, "bound": "hbm", "achieved": round(ach, 2), "peak": hbm, "unit": "GB/s",
           "frac": round(ach / hbm, 4), "traffic": None,
           "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6800 GB/s"}
    per_launch = v["bytes"] / max(v["launches"], 1)
    ratio = TRAFFIC_PER_ALGORITHMIC_BYTE.get(name)
    if ratio is not None:
        # DRAM bytes per launch from one ncu capture (profiles/), scaled by the
        # algorithmic bytes of this run's average launch
        out["traffic"] = round(ratio * per_launch)
        out["algorithmic_bytes_per_launch"] = round(per_launch)
    if name in ("tpanel", "tselect64") and n and exchange_us:
        floor_us, units, panels = panel_floor(n, exchange_us)
        facts = max(v["launches"], 1) / panels  # factorisations in the timed region
        ach_unit = 1e3 * v["ms"] / facts / units
        floor_unit = floor_us / units
        hbm_part = {k: out[k] for k in ("achieved", "peak", "unit", "frac", "traffic")}
        out = {"kernel": name, "bound": "latency", "achieved": round(ach_unit, 3), "peak": round(floor_unit, 3),
               "unit": "us per pivot group of 8 columns", "frac": round(floor_unit / ach_unit, 4),
               "traffic": hbm_part["traffic"],
               "floor": ("per group: max(one cluster exchange round of 8 nominees (2176 bytes) at the panel's "
                         "cluster size, measured by bola_measure_cluster_exchange; the group's FP32 work per CTA "
                         "at 128 FMA/clock/SM)"),
               "exchange_round_us": {str(c): round(exchange_us(c, 8 * TSLOT_BYTES), 3) for c in (2, 4, 8, 16)},
               "factorisations": round(facts, 2), "hbm": hbm_part}
        if name == "tpanel":
            out["note"] = ("launches of an abandoned 3xTF32 factorisation return at once and are averaged in, "
                           "so the time per group of the factorisations that ran is somewhat higher")
    return out


# ---------------------------------------------------------------- CPU ----

def cpu_solve_once(A_np, b_np):
    import oracle
    A = A_np.copy(order="F")
    B = b_np.copy(order="F")
    t0 = time.perf_counter()
    info, _ = oracle.solve_lu(A, B)
    dt = time.perf_counter() - t0
    if info != 0:
        raise RuntimeError(f"oracle getrf info {info}")
    return dt, B


def host_system(sysd, n, nrhs):
    A = sysd["A"].cpu().numpy().reshape(n, n).T  # column-major view -> F-ordered array
    b = sysd["b"].cpu().numpy().reshape(nrhs, n).T
    return np.asfortranarray(A), np.asfortranarray(b)


def cpu_baseline(sysd, n, nrhs, budget_s):
    """BOLA restated in C (oracle/) on all host threads, a bounded sample of
    complete n x n solves (at least one)."""
    import oracle
    oracle.lib()
    threads = oracle.get_threads()
    A, b = host_system(sysd, n, nrhs)
    times = []
    while True:
        dt, _ = cpu_solve_once(A, b)
        times.append(dt)
        if sum(times) + dt > budget_s:
            break
    v = len(times) / sum(times)
    return {"value": round(v, 5), "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": f"{len(times)} complete solve(s) n={n} nrhs={nrhs} (getrf + laswp + 2 trsm), kappa=1e2; "
                      f"BOLA restated in C (Rust not available to build BOLA)"}


def run_reference(args, device):
    import oracle
    n, nrhs = args.n, args.nrhs
    oracle.lib()
    systems = make_systems(n, nrhs, device)
    host = [host_system(s, n, nrhs) for s in systems]
    del systems
    torch.cuda.empty_cache()
    threads = oracle.get_threads()
    # warm-up solves (the first one also sizes the run: about 150 s of timed solves at most)
    warm = max(1, min(args.warmup, 5))
    t_warm = min(cpu_solve_once(*host[k % len(host)])[0] for k in range(warm))
    steps = max(1, min(args.steps, int(150.0 / max(t_warm, 1e-3))))
    per = []
    for k in range(steps):
        dt, _ = cpu_solve_once(*host[k % len(host)])
        per.append(dt)
    total = sum(per)
    value = steps / total
    sample = (f"{steps} complete solve(s) n={n} nrhs={nrhs} rotating kappa (getrf + laswp + 2 trsm) after {warm} "
              f"warm-up solve(s); "
              f"BOLA restated in C on {threads} host threads")
    return {
        "metric": METRIC, "impl": "reference", "value": round(value, 5), "unit": "solves/s", "n_gpus": 1,
        "steps": steps, "warmup": warm, "ms_per_step": round(1e3 * total / steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic, same systems as --impl ours",
        "config": {"workload": f"dense LU solve n={n} nrhs={nrhs} (BOLA getrf + laswp + 2 trsm), "
                               f"backward error <= {BERR_TARGET:g}",
                   "path": "BOLA's CPU algorithm (C restatement, OpenMP in place of Rayon)"},
        "latency_ms": {"p50": round(1e3 * statistics.median(per), 3),
                       "p99": round(1e3 * float(np.percentile(per, 99)), 3)},
        "cpu_baseline": {"value": round(value, 5), "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 5), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        out = run_reference(args, torch.device("cuda", local))
        print(json.dumps(out), flush=True)
        return 0
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    if world > 1:
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.distributed.init_process_group("nccl", device_id=device)
    out = run_ours(args, rank, world, device)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
