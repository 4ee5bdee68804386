"""Continuous-batching solve server on one GPU.

Requests (PDE kind, grid size, batch, step count, dt, initial field) arrive
over time. Requests of the same kind and grid size share a *bucket*: one
plan whose coefficient tables have one entry per slot (each slot carries its
own dt, set with ``fsm_plan_set_batch_dt``), one slot-batched spectral state
and one workspace, sized at start-up from an HBM budget. Every *tick*
advances all active slots of a bucket by up to ``chunk`` steps in one fused
launch sequence (2D: one column + one row pass launch per stage for all
slots; 1D: one launch); buckets tick on their own streams, so their work
overlaps on the device. Between ticks finished requests leave (their slots
are transformed back and copied to the host), the remaining slots are
compacted, and waiting requests are admitted while slots are free.

Per-sample arithmetic is independent of the other samples in the launch,
so a request's result is the same alone and in the mix.

The reference has no serving layer; the solves themselves follow
``Operator.integrate`` (operator/_base.py:676-751) for
``KuramotoSivashinsky()`` (pde.py:27-39) and ``Burgers(nu)`` (pde.py:13-25).
"""

from __future__ import annotations

import collections
import math
import threading
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np
import torch

from . import _lib, _native, pde
from .mesh import FourierMesh

KS_LENGTH = 32 * math.pi
BURGERS_NU = 0.01


@dataclass
class SolveRequest:
    rid: int
    kind: str            # "ks1d" | "burgers2d"
    n: int
    batch: int
    steps: int
    dt: float
    u0: torch.Tensor     # host float32 [batch, C, *shape]
    arrival: float = 0.0
    t_admit: Optional[float] = None
    t_done: Optional[float] = None
    result: Optional[torch.Tensor] = None
    remaining: int = 0
    slots: List[int] = field(default_factory=list)

    @property
    def dof_steps(self) -> int:
        return int(np.prod(self.u0.shape)) * self.steps


def problem(kind: str, n: int):
    """(operator, mesh_info, channels) of a request kind."""
    if kind == "ks1d":
        return pde.KuramotoSivashinsky(), [(0.0, KS_LENGTH, n)], 1
    if kind == "burgers2d":
        return pde.Burgers(BURGERS_NU), [(0.0, 2 * math.pi, n), (0.0, 2 * math.pi, n)], 2
    raise ValueError(kind)


def slot_bytes(kind: str, n: int, chunk: int) -> int:
    """HBM per slot: state + workspace + coefficient tables."""
    _, mesh, C = problem(kind, n)
    shape = [m[2] for m in mesh]
    S = int(np.prod(shape[:-1])) * (shape[-1] // 2 + 1)
    per_field = S * 8
    if kind == "ks1d":
        return per_field * (C + 6)
    return per_field * (C + 2 * C + 4 + C + 6)


# Ticks of at most GRAPH_MAX_STEPS steps replay a CUDA graph captured per (active slots, steps);
# the step count of such ticks is rounded down to a power of two so that few shapes recur.
GRAPH_MAX_STEPS = 64
GRAPH_CACHE = 48


class _Bucket:
    def __init__(self, kind: str, n: int, capacity: int, device: torch.device, chunk: int,
                 priority: int = 0, tick_ms: float = 4.0, graphs: bool = True):
        self.kind, self.n, self.capacity, self.device, self.chunk = kind, n, capacity, device, chunk
        self.tick_ms = tick_ms
        self.use_graphs = graphs
        self.graphs: "collections.OrderedDict[Tuple[int, int], torch.cuda.CUDAGraph]" = collections.OrderedDict()
        self._seen: set = set()
        self.replays = 0
        self.step_ms: Optional[float] = None  # measured device time per step and slot
        op, mesh, C = problem(kind, n)
        self.C = C
        f_mesh = FourierMesh(mesh, device=device, dtype=torch.float32)
        op.register_mesh(f_mesh, C)
        prog = _native.lower(op._linear_terms, op._nonlinear_funcs, f_mesh, C, op._de_aliasing_rate)
        self.stream = torch.cuda.Stream(device, priority=priority)
        with torch.cuda.stream(self.stream):
            self.plan = _native.NativePlan(prog, 0.05, _lib.FSM_SETDRK4, device,
                                           linear_coef64=op._linear_coef64(device), table_batch=capacity)
            self.sp = _native.Spectral(self.plan)
            half = tuple(m[2] for m in mesh[:-1]) + (mesh[-1][2] // 2 + 1,)
            self.state = torch.empty((capacity, C) + half, dtype=torch.complex64, device=device)
            self.ws = torch.empty(self.plan.workspace_bytes(capacity, chunk), dtype=torch.uint8, device=device)
        self.owner: List[Optional[Tuple[SolveRequest, int]]] = [None] * capacity
        self.active: List[SolveRequest] = []
        self.n_active = 0
        self.tick: Optional[Tuple[torch.cuda.Event, torch.cuda.Event, int, int]] = None
        self.launches = 0

    def can_admit(self, req: SolveRequest) -> bool:
        return self.tick is None and self.capacity - self.n_active >= req.batch

    def admit(self, req: SolveRequest, now: float) -> None:
        with torch.cuda.stream(self.stream):
            u = req.u0.to(self.device, non_blocking=True)
            half = self.sp.to_half(u)
            lo = self.n_active
            self.state[lo:lo + req.batch].copy_(half)
            for i in range(req.batch):
                self.plan.set_batch_dt(lo + i, req.dt)
                self.owner[lo + i] = (req, i)
        req.slots = list(range(lo, lo + req.batch))
        req.remaining = req.steps
        req.t_admit = now
        self.active.append(req)
        self.n_active += req.batch

    def launch(self) -> None:
        k = min(self.chunk, min(r.remaining for r in self.active))
        if self.step_ms:
            # ticks of about tick_ms of device work keep admission and small requests responsive
            k = max(1, min(k, int(self.tick_ms / (self.step_ms * self.n_active))))
        if self.use_graphs and k <= GRAPH_MAX_STEPS:
            k = 1 << (k.bit_length() - 1)
        with torch.cuda.stream(self.stream):
            e0 = torch.cuda.Event(enable_timing=True)
            e0.record(self.stream)
            self._advance(self.n_active, k)
            e1 = torch.cuda.Event(enable_timing=True)
            e1.record(self.stream)
        # a captured tick (graph replay) runs one launch sequence; a direct one may run in parts
        graphed = self.use_graphs and k <= GRAPH_MAX_STEPS and (self.n_active, k) in self.graphs
        self.launches += self.plan.launch_count(k, 0 if graphed else self.n_active)
        self.tick = (e0, e1, k, self.n_active)

    def _advance(self, n: int, k: int) -> None:
        """k steps of slots [0, n) on the bucket's stream (the current stream here): a replay of the
        graph of (n, k) when there is one. A shape is captured the second time it occurs (the first
        run sets the kernels' attributes); the capture is thread-local, so the other buckets' host
        threads keep launching meanwhile."""
        if not self.use_graphs or k > GRAPH_MAX_STEPS:
            self.plan.integrate_half(self.state[:n], k, workspace=self.ws)
            return
        key = (n, k)
        g = self.graphs.get(key)
        if g is None:
            if key not in self._seen:
                self._seen.add(key)
                self.plan.integrate_half(self.state[:n], k, workspace=self.ws)
                return
            g = torch.cuda.CUDAGraph()
            g.capture_begin(capture_error_mode="thread_local")
            try:
                self.plan.integrate_half(self.state[:n], k, workspace=self.ws)
            finally:
                g.capture_end()
            self.graphs[key] = g
            while len(self.graphs) > GRAPH_CACHE:
                self.graphs.popitem(last=False)
        else:
            self.graphs.move_to_end(key)
        g.replay()
        self.replays += 1

    def poll(self) -> List[SolveRequest]:
        """Finish the tick if the device is done with it; return the requests that completed, whose
        results are being copied to pinned host memory (``r._copied`` records when)."""
        if self.tick is None or not self.tick[1].query():
            return []
        e0, e1, k, n = self.tick
        self.tick = None
        ms = e0.elapsed_time(e1) / (k * n)
        self.step_ms = ms if self.step_ms is None else 0.5 * (self.step_ms + ms)
        done = []
        for r in self.active:
            r.remaining -= k
            if r.remaining == 0:
                done.append(r)
        if not done:
            return []
        with torch.cuda.stream(self.stream):
            for r in done:
                idx = torch.tensor(r.slots, device=self.device)
                out = self.sp.to_physical(self.state.index_select(0, idx), keep_input=False)
                r.result = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)
                r.result.copy_(out, non_blocking=True)
                r._copied = torch.cuda.Event()
                r._copied.record(self.stream)
        for r in done:
            for s in r.slots:
                self.owner[s] = None
        self.active = [r for r in self.active if r.remaining > 0]
        self._compact()
        return done

    def _compact(self) -> None:
        """Move the highest occupied slots into freed holes so that slots [0, n_active) are occupied."""
        occupied = [i for i in range(self.capacity) if self.owner[i] is not None]
        n = len(occupied)
        holes = [i for i in range(n) if self.owner[i] is None]
        movers = [i for i in occupied if i >= n]
        with torch.cuda.stream(self.stream):
            for h, m in zip(holes, movers):
                self.state[h].copy_(self.state[m])
                self.plan.move_batch(h, m)
                req, i = self.owner[m]
                req.slots[i] = h
                self.owner[h] = (req, i)
                self.owner[m] = None
        self.n_active = n


class SolveServer:
    """Admission by HBM budget, per-bucket ticks on separate streams."""

    def __init__(self, device: torch.device, hbm_budget_bytes: int = 8 << 30, chunk: int = 50,
                 max_slots: int = 256, tick_ms: float = 4.0, graphs: bool = True, priority: str = "cheap"):
        """``priority``: which buckets get the high-priority streams, "cheap" (1D and 64^2 grids,
        whose requests are short) or "costly" (the large 2D grids, whose requests are the long tail)."""
        self.device = device
        self.graphs = graphs
        self.priority = priority
        self.budget = hbm_budget_bytes
        self.chunk = chunk
        self.max_slots = max_slots
        self.tick_ms = tick_ms
        self.buckets: Dict[Tuple[str, int], _Bucket] = {}

    def prepare(self, keys: List[Tuple[str, int]], max_batch: int = 32) -> None:
        """Create one bucket per (kind, n), splitting the HBM budget by footprint."""
        share = self.budget // max(1, len(keys))
        lo, hi = torch.cuda.Stream.priority_range()
        for kind, n in keys:
            cap = int(min(self.max_slots, max(max_batch, share // slot_bytes(kind, n, self.chunk))))
            cheap = kind == "ks1d" or n <= 64
            prio = hi if cheap == (self.priority == "cheap") else lo
            self.buckets[(kind, n)] = _Bucket(kind, n, cap, self.device, self.chunk, prio, self.tick_ms, self.graphs)
        torch.cuda.synchronize(self.device)

    def run(self, requests: List[SolveRequest], realtime: bool = True) -> float:
        """Serve the requests (arrival times in seconds from start); returns the wall time."""
        pending = sorted(requests, key=lambda r: r.arrival)
        keys = sorted({(r.kind, r.n) for r in pending})
        missing = [k for k in keys if k not in self.buckets]
        if missing:
            self.prepare(missing)
        waiting: Dict[Tuple[str, int], collections.deque] = {k: collections.deque() for k in self.buckets}
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        i, finished, total = 0, 0, len(pending)
        copying: List[SolveRequest] = []
        while finished < total:
            t = now()
            while i < total and (not realtime or pending[i].arrival <= t):
                waiting[(pending[i].kind, pending[i].n)].append(pending[i])
                i += 1
            busy = bool(copying)
            still = []
            for r in copying:
                if r._copied.query():
                    r.t_done = now()
                    finished += 1
                else:
                    still.append(r)
            copying = still
            for key, b in self.buckets.items():
                copying.extend(b.poll())
                if b.tick is None:
                    q = waiting[key]
                    while q and b.can_admit(q[0]):
                        b.admit(q.popleft(), now())
                    if b.n_active:
                        b.launch()
                if b.tick is not None:
                    busy = True
            if not busy:
                time.sleep(0.0001)
        return now()

    def run_threaded(self, requests: List[SolveRequest], realtime: bool = True) -> float:
        """Serve with one host worker thread per bucket: each worker admits, launches its bucket's
        ticks and waits for them (the library calls and event waits release the GIL), so host-side
        launch work of different buckets overlaps. The main thread releases requests at their
        arrival times. Returns the wall time."""
        pending = sorted(requests, key=lambda r: r.arrival)
        keys = sorted({(r.kind, r.n) for r in pending})
        missing = [k for k in keys if k not in self.buckets]
        if missing:
            self.prepare(missing)
        queues = {k: collections.deque() for k in self.buckets}
        cond = threading.Condition()
        state = {"arrived": False}
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        device = self.device
        errors: List[BaseException] = []

        def worker(key):
            b = self.buckets[key]
            q = queues[key]
            try:
                with torch.cuda.device(device):
                    while True:
                        with cond:
                            while not q and b.n_active == 0 and not state["arrived"]:
                                cond.wait(0.01)
                            batch = []
                            while q and b.capacity - b.n_active - sum(r.batch for r in batch) >= q[0].batch:
                                batch.append(q.popleft())
                            finished = state["arrived"] and not q and b.n_active == 0 and not batch
                        if finished:
                            return
                        for r in batch:
                            b.admit(r, now())
                        if b.n_active == 0:
                            continue
                        b.launch()
                        b.tick[1].synchronize()
                        for r in b.poll():
                            r._copied.synchronize()
                            r.t_done = now()
            except BaseException as e:  # surface worker failures to the caller
                errors.append(e)

        threads = [threading.Thread(target=worker, args=(k,), daemon=True) for k in self.buckets]
        for th in threads:
            th.start()
        for r in pending:
            if realtime:
                delay = r.arrival - now()
                if delay > 0:
                    time.sleep(delay)
            with cond:
                queues[(r.kind, r.n)].append(r)
                cond.notify_all()
        with cond:
            state["arrived"] = True
            cond.notify_all()
        for th in threads:
            th.join()
        if errors:
            raise errors[0]
        return now()

    @property
    def launches(self) -> int:
        return sum(b.launches for b in self.buckets.values())

    @property
    def graph_replays(self) -> int:
        return sum(b.replays for b in self.buckets.values())


def make_stream(count: int, seed: int, rate_hz: float, max_steps: int = 2000, min_steps: int = 100,
                kmax: int = 8) -> List[SolveRequest]:
    """The mixed request stream: uniform over {KS 1D, N in 256..4096; 2D Burgers, N in 64..256},
    batch 1-32, steps 100-2000, dt 0.01-0.1, band-limited N(0,1) initial fields (|k| <= 8) scaled to
    RMS 1 (KS) / 0.25 (Burgers: unit RMS diverges at dt >= 0.02 in the reference), Poisson arrivals."""
    from . import initial

    rng = np.random.Generator(np.random.PCG64(seed))
    # arrival gaps come from their own generator, so that the requests (kind, size, batch, steps,
    # dt, initial field) are the same at every rate and a stream can be compared request by request
    # with its burst (rate 0) or one-at-a-time run
    arrivals = np.random.Generator(np.random.PCG64([seed, 1]))
    t = 0.0
    out = []
    for rid in range(count):
        t += arrivals.exponential(1.0 / rate_hz) if rate_hz > 0 else 0.0
        if rng.integers(0, 2) == 0:
            kind, n, rms = "ks1d", int(rng.choice([256, 512, 1024, 2048, 4096])), 1.0
            shape = (n,)
            C = 1
        else:
            kind, n, rms = "burgers2d", int(rng.choice([64, 128, 256])), 0.25
            shape = (n, n)
            C = 2
        batch = int(rng.integers(1, 33))
        steps = int(rng.integers(min_steps, max_steps + 1))
        dt = float(rng.uniform(0.01, 0.1))
        u0 = initial.band_limited(shape, batch, C, kmax, int(rng.integers(0, 2 ** 31)), rms).astype(np.float32)
        out.append(SolveRequest(rid, kind, n, batch, steps, dt, torch.from_numpy(u0), arrival=t))
    return out


def solve_alone(req: SolveRequest, device: torch.device, ops: Dict) -> Tuple[torch.Tensor, float]:
    """The plain drop-in: one ``integrate`` call for the request, result copied to the host."""
    key = (req.kind, req.n)
    if key not in ops:
        ops[key] = problem(req.kind, req.n)
    op, mesh, _ = ops[key]
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    u = req.u0.to(device)
    out = op.integrate(u_0=u, mesh=mesh if op._state_dict["f_mesh"] is None else None, dt=req.dt, step=req.steps)
    res = out.cpu()
    return res, time.perf_counter() - t0
