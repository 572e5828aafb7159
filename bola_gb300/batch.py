"""Batches of small independent systems for bola_batch_* (include/bola_gb300.h).

`Batch` packs the systems' matrices and right-hand sides into two device
buffers, builds the device array of `bola_system` descriptors, and owns the
plan (bucketing, group sizes, work order) created by the C library.
"""
import ctypes

import numpy as np
import torch

from . import _lib


class Batch:
    """A batch of systems A_i X_i = B_i on one device.

    ns, nrhs, kinds: per-system order, right-hand-side count and kind (0 LU,
    1 Cholesky).  tuning: a Tuning (the autotuner's output, or one loaded from
    its JSON file), or an 8-entry group-size table; None = library defaults.
    """

    def __init__(self, ns, nrhs, kinds, device="cuda", tuning=None):
        self.L = _lib.load()
        self.ns = np.asarray(ns, dtype=np.int32)
        self.nrhs = np.asarray(nrhs, dtype=np.int32)
        self.kinds = np.asarray(kinds, dtype=np.int32)
        self.count = len(self.ns)
        self.a_off = np.zeros(self.count + 1, dtype=np.int64)
        self.a_off[1:] = np.cumsum(self.ns.astype(np.int64) ** 2)
        self.b_off = np.zeros(self.count + 1, dtype=np.int64)
        self.b_off[1:] = np.cumsum(self.ns.astype(np.int64) * self.nrhs)
        self.A = torch.empty(int(self.a_off[-1]), dtype=torch.float64, device=device)
        self.B = torch.empty(int(self.b_off[-1]), dtype=torch.float64, device=device)
        self.info = torch.zeros(self.count, dtype=torch.int32, device=device)
        desc = (_lib.System * max(self.count, 1))()
        a0, b0 = self.A.data_ptr(), self.B.data_ptr()
        for i in range(self.count):
            n = int(self.ns[i])
            desc[i] = _lib.System(n, int(self.nrhs[i]), int(self.kinds[i]), n, n, 0, a0 + 8 * int(self.a_off[i]),
                                  b0 + 8 * int(self.b_off[i]))
        raw = np.frombuffer(desc, dtype=np.uint8)
        self.desc = torch.from_numpy(raw.copy()).to(device)
        self.plan = ctypes.c_void_p()
        self.replan(tuning)

    def replan(self, tuning=None):
        """(Re)build the plan with a Tuning, an 8-entry group-size table, or the defaults (None)."""
        self.close()
        if tuning is not None and not isinstance(tuning, Tuning):
            tuning = Tuning(group_size=tuning)
        self.tuning = tuning
        st = self.L.bola_batch_plan_create_tuned(self.count, self.ns.ctypes.data_as(ctypes.c_void_p),
                                                 self.kinds.ctypes.data_as(ctypes.c_void_p),
                                                 ctypes.byref(tuning.c()) if tuning is not None else None,
                                                 ctypes.byref(self.plan))
        if st != 0:
            raise RuntimeError(f"bola_batch_plan_create: {st} {self.L.bola_last_error().decode()}")

    def a_view(self, i):
        n = int(self.ns[i])
        return self.A[int(self.a_off[i]):int(self.a_off[i + 1])].view(n, n).t()  # column-major n x n

    def b_view(self, i):
        n, r = int(self.ns[i]), int(self.nrhs[i])
        return self.B[int(self.b_off[i]):int(self.b_off[i + 1])].view(r, n).t()

    def flops(self):
        f = ctypes.c_double()
        self.L.bola_batch_plan_info(self.plan, None, None, ctypes.byref(f))
        return f.value

    def solve(self, graph=False, stream=None):
        s = ctypes.c_void_p((stream or torch.cuda.current_stream()).cuda_stream)
        fn = self.L.bola_batch_solve_graph if graph else self.L.bola_batch_solve
        st = fn(self.plan, ctypes.c_void_p(self.desc.data_ptr()), ctypes.c_void_p(self.info.data_ptr()), s)
        if st != 0:
            raise RuntimeError(f"bola_batch_solve: {st} {self.L.bola_last_error().decode()}")

    def close(self):
        if self.plan:
            self.L.bola_batch_plan_destroy(self.plan)
            self.plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def config4_batch(count, seed=4, device="cuda", nmin=8, nmax=256, rmax=8):
    """The batched-solve workload: n uniform-integer in [nmin, nmax], even ids
    LU on uniform[-1,1) + n*I, odd ids Cholesky on B B^T / n + I (B uniform
    [-1,1)), nrhs uniform in [1, rmax], right-hand sides uniform [-1,1).
    Returns (ns, nrhs, kinds, fill) where fill(batch) writes the matrices."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(nmin, nmax + 1, size=count).astype(np.int32)
    nrhs = rng.integers(1, rmax + 1, size=count).astype(np.int32)
    kinds = (np.arange(count) % 2).astype(np.int32)

    def fill(batch):
        g = torch.Generator(device=device)
        g.manual_seed(seed)
        for i in range(count):
            n = int(ns[i])
            M = torch.rand(n, n, dtype=torch.float64, device=device, generator=g) * 2 - 1
            if kinds[i] == 0:
                M += n * torch.eye(n, dtype=torch.float64, device=device)
            else:
                M = M @ M.t() / n + torch.eye(n, dtype=torch.float64, device=device)
            batch.a_view(i).copy_(M)
            batch.b_view(i).copy_(torch.rand(n, int(nrhs[i]), dtype=torch.float64, device=device, generator=g) * 2 - 1)
    return ns, nrhs, kinds, fill


BUCKET_N = (16, 32, 48, 64, 96, 128, 192, 256)
DEFAULT_GROUPS = (32, 32, 64, 64, 128, 128, 256, 256)
GROUP_CHOICES = (32, 64, 128, 256)
PANEL_CHOICES = (8, 12, 16)
TILE_CHOICES = (4, 2)


class Tuning:
    """The batched solver's tuning table (bola_batch_tuning): per size bucket
    the group size and the panel width, and one register-tile height."""

    def __init__(self, group_size=None, panel_width=None, tile_rows=4):
        self.group_size = [int(v) for v in (group_size or DEFAULT_GROUPS)]
        self.panel_width = [int(v) for v in (panel_width or (8,) * 8)]
        self.tile_rows = int(tile_rows)

    def c(self):
        return _lib.BatchTuning((ctypes.c_int32 * 8)(*self.group_size), (ctypes.c_int32 * 8)(*self.panel_width),
                                self.tile_rows, 0)

    def as_dict(self):
        return {"group_size": self.group_size, "panel_width": self.panel_width, "tile_rows": self.tile_rows}

    def save(self, path):
        """Writes the table as JSON through the library (bola_batch_tuning_save)."""
        st = _lib.load().bola_batch_tuning_save(str(path).encode(), ctypes.byref(self.c()))
        if st != 0:
            raise RuntimeError(f"bola_batch_tuning_save: {st} {_lib.load().bola_last_error().decode()}")

    @classmethod
    def load(cls, path):
        """Reads a table written by save (bola_batch_tuning_load); returns (Tuning, SM count it was measured on)."""
        t, sms = _lib.BatchTuning(), ctypes.c_int32()
        st = _lib.load().bola_batch_tuning_load(str(path).encode(), ctypes.byref(t), ctypes.byref(sms))
        if st != 0:
            raise ValueError(f"bola_batch_tuning_load: {st} {_lib.load().bola_last_error().decode()}")
        return cls(list(t.group_size), list(t.panel_width), t.tile_rows or 4), sms.value


def bucket_of(n):
    for b, top in enumerate(BUCKET_N):
        if n <= top:
            return b
    raise ValueError(n)


def time_solve(batch, A0, B0, reps, graph=True):
    """Minimum CUDA-event time (ms) of one batched solve over `reps` runs, the
    inputs restored from A0/B0 before each (outside the timed region)."""
    stream = torch.cuda.current_stream()
    best = float("inf")
    for _ in range(reps):
        batch.A.copy_(A0)
        batch.B.copy_(B0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.solve(graph=graph)
        e1.record(stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def autotune(batch, reps=3, path=None):
    """Per size bucket, the (group size, panel width) pair with the shortest
    solve of that bucket's systems of `batch` (a sub-batch holding copies of
    them), then the register tile with the shortest solve of the whole batch
    under that table.  Every choice leaves each system's operation order
    unchanged (results are bit-identical), so only time decides.  Writes the
    table to `path` as JSON if given.  Returns (Tuning, trials), trials =
    {bucket: {"G/PB": ms}, "tile": {rows: ms}}."""
    buckets = np.array([bucket_of(int(n)) for n in batch.ns])
    best = Tuning()
    trials = {}
    for b in range(len(BUCKET_N)):
        idx = np.nonzero(buckets == b)[0]
        if len(idx) == 0:
            continue
        sub = Batch(batch.ns[idx], batch.nrhs[idx], batch.kinds[idx], device=batch.A.device)
        for j, i in enumerate(idx):
            sub.a_view(j).copy_(batch.a_view(int(i)))
            sub.b_view(j).copy_(batch.b_view(int(i)))
        A0, B0 = sub.A.clone(), sub.B.clone()
        trials[b] = {}
        for g in GROUP_CHOICES:
            for pw in PANEL_CHOICES:
                t = Tuning(best.group_size, best.panel_width, best.tile_rows)
                t.group_size[b], t.panel_width[b] = g, pw
                sub.replan(t)
                sub.solve(graph=False)  # warm-up
                trials[b][f"{g}/{pw}"] = time_solve(sub, A0, B0, reps, graph=False)
        g, pw = min(trials[b], key=trials[b].get).split("/")
        best.group_size[b], best.panel_width[b] = int(g), int(pw)
        sub.close()
    A0, B0 = batch.A.clone(), batch.B.clone()
    trials["tile"] = {}
    for tr in TILE_CHOICES:
        t = Tuning(best.group_size, best.panel_width, tr)
        batch.replan(t)
        batch.solve(graph=False)
        trials["tile"][tr] = time_solve(batch, A0, B0, reps, graph=False)
    best.tile_rows = min(trials["tile"], key=trials["tile"].get)
    batch.A.copy_(A0)
    batch.B.copy_(B0)
    batch.replan(best)
    if path is not None:
        best.save(path)
    return best, trials
