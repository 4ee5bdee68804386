"""Continuous-batching solve server on one GPU.

Requests (PDE kind, grid size, batch, step count, dt, initial field) arrive
over time. Requests of the same kind and grid size share a *bucket*: one
plan whose coefficient tables have one entry per slot (each slot carries its
own dt) and the library's serving engine (``fsm_serve_*``, csrc/fsm_serve.cu)
over one slot-batched spectral state and one workspace, sized at start-up
from an HBM budget. The engine runs the scheduling in native code: every
*tick* admits waiting requests while slots are free, then advances all
occupied slots by up to ``chunk`` steps in one fused launch sequence (2D: one
column + one row pass launch per stage for all slots; 1D: one launch), short
ticks replayed as CUDA graphs; when a tick completes, finished requests write
their slots back and leave, and the remaining slots are compacted. Buckets
tick on their own streams, so their work overlaps on the device. Python turns
requests into half spectra and results back into fields on the host.

Per-sample arithmetic is independent of the other samples in the launch,
so a request's result is the same alone and in the mix.

The reference has no serving layer; the solves themselves follow
``Operator.integrate`` (operator/_base.py:676-751) for
``KuramotoSivashinsky()`` (pde.py:27-39) and ``Burgers(nu)`` (pde.py:13-25).
"""

from __future__ import annotations

import collections
import gc
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

    @property
    def finite(self) -> Optional[bool]:
        """False when the result holds NaN or Inf (the solve diverged), None before the result has
        reached the host. Read it once ``t_done`` is set: the result is copied asynchronously."""
        if self.result is None or self.t_done is None:
            return None
        return bool(torch.isfinite(self.result).all())


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


# Ticks of at most GRAPH_MAX_STEPS steps replay a CUDA graph captured per (occupied slots, steps);
# the step count of such ticks is rounded down to a power of two so that few shapes recur
# (the library's serving engine, fsm_serve_tick).
GRAPH_MAX_STEPS = 64
# Requests handed to a bucket's engine ahead of admission (their half spectra wait on the device).
ENGINE_QUEUE = 4


class _Bucket:
    """One (kind, n): a plan with one table entry per slot and the library's serving engine
    (``fsm_serve_*``: admission, ticks, completion, slot compaction and graph replay run in
    native code on the bucket's stream). Python transforms requests in and out of the half
    spectrum and copies results to pinned host memory."""

    def __init__(self, kind: str, n: int, capacity: int, device: torch.device, chunk: int,
                 priority: int = 0, tick_ms: float = 4.0, graphs: bool = True,
                 stream: Optional[torch.cuda.Stream] = None):
        self.kind, self.n, self.capacity, self.device, self.chunk = kind, n, capacity, device, chunk
        op, mesh, C = problem(kind, n)
        self.C = C
        f_mesh = FourierMesh(mesh, device=device, dtype=torch.float32)
        op.register_mesh(f_mesh, C)
        prog = _native.lower(op._linear_terms, op._nonlinear_funcs, f_mesh, C, op._de_aliasing_rate)
        self.stream = stream if stream is not None else torch.cuda.Stream(device, priority=priority)
        with torch.cuda.stream(self.stream):
            self.plan = _native.NativePlan(prog, 0.05, _lib.FSM_SETDRK4, device,
                                           linear_coef64=op._linear_coef64(device), table_batch=capacity)
            self.sp = _native.Spectral(self.plan)
        self.engine = _native.ServePool(self.plan, capacity, chunk, self.stream, graphs=graphs, tick_ms=tick_ms)
        self.pending: Dict[int, SolveRequest] = {}  # submitted to the engine, not yet completed
        self.in_flight = False

    def submit(self, req: SolveRequest, now: float) -> None:
        """Hand a request to the engine (it is admitted into slots at the engine's next tick)."""
        with torch.cuda.stream(self.stream):
            u = req.u0.to(self.device, non_blocking=True)
            req._half = self.sp.to_half(u).contiguous()
        self.engine.submit(req.rid, req.steps, req.dt, req._half)
        req.t_admit = now
        req.remaining = req.steps
        self.pending[req.rid] = req

    def feed(self, queue: "collections.deque", now: float) -> None:
        """Submit queued requests while the engine holds fewer than ENGINE_QUEUE waiting ones."""
        waiting = self.engine.stats()["waiting"] if queue else 0
        while queue and waiting < ENGINE_QUEUE:
            self.submit(queue.popleft(), now)
            waiting += 1

    def launch(self) -> int:
        """The engine's next tick (admission + k steps of every occupied slot); k, 0 when idle or busy."""
        k = self.engine.tick()
        if k:
            self.in_flight = True
        return k

    def poll(self, wait: bool = False) -> List[SolveRequest]:
        """Complete the tick if the device is done with it; return the requests that completed, whose
        results are being copied to pinned host memory (``r._copied`` records when)."""
        if not self.in_flight:
            return []
        ids, self.in_flight = self.engine.poll(wait)
        return self.finish(ids)

    def finish(self, ids: List[int]) -> List[SolveRequest]:
        """Turn the completed requests' half spectra into fields and start their copies to pinned host
        memory on the bucket's stream."""
        done = []
        with torch.cuda.stream(self.stream):
            for rid in ids:
                r = self.pending.pop(rid)
                out = self.sp.to_physical(r._half, keep_input=False)
                r._half = None
                r.remaining = 0
                r.result = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)
                r.result.copy_(out, non_blocking=True)
                r._copied = torch.cuda.Event()
                r._copied.record(self.stream)
                done.append(r)
        return done

    def close(self) -> None:
        """Destroy the engine (it waits for the bucket's stream), then the plan it used."""
        if self.engine is not None:
            self.engine.__del__()
            self.engine = None
        if self.plan is not None:
            self.plan.__del__()
            self.plan = None

    @property
    def idle(self) -> bool:
        st = self.engine.stats()
        return not self.in_flight and st["occupied"] == 0 and st["waiting"] == 0

    @property
    def launches(self) -> int:
        return self.engine.stats()["launches"]

    @property
    def replays(self) -> int:
        return self.engine.stats()["graph_replays"]


class _Group:
    """Buckets ticked together by the library's serving group (``fsm_serve_group_*``): every tick
    advances every occupied slot of every member by the same number of steps. The 1D KS buckets
    (every grid size) form one group whose tick is ONE launch of the line kernel; the 2D Burgers
    buckets (64^2, 128^2, 256^2) one group whose column and row passes are one launch each per
    stage. The members share one stream."""

    def __init__(self, buckets: List[_Bucket], tick_ms: float):
        self.buckets = buckets
        self.stream = buckets[0].stream
        self.group = _native.ServeGroup([b.engine for b in buckets], tick_ms=tick_ms)
        self.in_flight = False

    def feed(self, queues: Dict[Tuple[str, int], "collections.deque"], now: float) -> None:
        for b in self.buckets:
            b.feed(queues[(b.kind, b.n)], now)

    def launch(self) -> int:
        k = self.group.tick()
        if k:
            self.in_flight = True
        return k

    def poll(self, wait: bool = False) -> List[SolveRequest]:
        if not self.in_flight:
            return []
        self.in_flight = self.group.poll(wait)
        if self.in_flight:
            return []
        done = []
        for b in self.buckets:
            ids, _ = b.engine.poll(False)
            done.extend(b.finish(ids))
        return done

    def close(self) -> None:
        """Release the group (it waits for the stream); the members are closed by their owner."""
        if self.group is not None:
            self.group.close()
            self.group = None

    @property
    def idle(self) -> bool:
        return not self.in_flight and all(b.idle for b in self.buckets)

    @property
    def launches(self) -> int:
        return self.group.stats()["launches"] if self.group is not None else 0


class SolveServer:
    """Admission by HBM budget, per-bucket ticks on separate streams."""

    def __init__(self, device: torch.device, hbm_budget_bytes: int = 8 << 30, chunk: int = 50,
                 max_slots: int = 256, tick_ms: float = 4.0, graphs: bool = True, priority: str = "cheap",
                 group_lines: bool = True, group_planes: bool = False):
        """``priority``: which buckets get the high-priority streams, "cheap" (1D and 64^2 grids,
        whose requests are short) or "costly" (the large 2D grids, whose requests are the long tail).
        ``group_lines``: the 1D KS buckets of every grid size advance together, one launch per tick.
        ``group_planes``: the 2D Burgers buckets of every grid size tick together on one stream."""
        self.device = device
        self.graphs = graphs
        self.priority = priority
        self.budget = hbm_budget_bytes
        self.chunk = chunk
        self.max_slots = max_slots
        self.tick_ms = tick_ms
        self.group_lines = group_lines
        self.group_planes = group_planes
        self.buckets: Dict[Tuple[str, int], _Bucket] = {}
        self.groups: List[_Group] = []

    def prepare(self, keys: List[Tuple[str, int]], max_batch: int = 32) -> None:
        """Create one bucket per (kind, n), splitting the HBM budget by footprint; the 1D KS buckets
        (with ``group_lines``) share one stream and one serving group."""
        share = self.budget // max(1, len(keys))
        lo, hi = torch.cuda.Stream.priority_range()
        line_keys = [k for k in keys if k[0] == "ks1d"] if self.group_lines else []
        plane_keys = [k for k in keys if k[0] == "burgers2d"] if self.group_planes else []
        shared = {}
        if len(line_keys) > 1:
            shared["line"] = torch.cuda.Stream(self.device, priority=hi if self.priority == "cheap" else lo)
        if len(plane_keys) > 1:
            shared["plane"] = torch.cuda.Stream(self.device, priority=lo if self.priority == "cheap" else hi)
        for kind, n in keys:
            cap = int(min(self.max_slots, max(max_batch, share // slot_bytes(kind, n, self.chunk))))
            cheap = kind == "ks1d" or n <= 64
            prio = hi if cheap == (self.priority == "cheap") else lo
            stream = shared.get("line") if (kind, n) in line_keys else shared.get("plane") if (kind, n) in plane_keys else None
            self.buckets[(kind, n)] = _Bucket(kind, n, cap, self.device, self.chunk, prio, self.tick_ms, self.graphs,
                                              stream=stream)
        for name, ks in (("line", line_keys), ("plane", plane_keys)):
            if name in shared:
                self.groups.append(_Group([self.buckets[k] for k in sorted(ks, key=lambda k: k[1])], self.tick_ms))
        torch.cuda.synchronize(self.device)

    def _units(self) -> list:
        """What the host loop ticks: every group, and every bucket outside a group."""
        grouped = {id(b) for g in self.groups for b in g.buckets}
        return list(self.groups) + [b for b in self.buckets.values() if id(b) not in grouped]

    def run(self, requests: List[SolveRequest], realtime: bool = True) -> float:
        """Serve the requests (arrival times in seconds from start); returns the wall time."""
        pending = sorted(requests, key=lambda r: r.arrival)
        keys = sorted({(r.kind, r.n) for r in pending})
        missing = [k for k in keys if k not in self.buckets]
        if missing:
            self.prepare(missing)
        waiting: Dict[Tuple[str, int], collections.deque] = {k: collections.deque() for k in self.buckets}
        units = self._units()
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
            for u in units:
                copying.extend(u.poll())
                if isinstance(u, _Group):
                    u.feed(waiting, t)
                else:
                    u.feed(waiting[(u.kind, u.n)], t)
                if not u.in_flight:
                    u.launch()
                if u.in_flight:
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

        def worker(u):
            grouped = isinstance(u, _Group)
            mine = [queues[(b.kind, b.n)] for b in u.buckets] if grouped else [queues[(u.kind, u.n)]]
            try:
                with torch.cuda.device(device):
                    while True:
                        with cond:
                            while not any(mine) and u.idle and not state["arrived"]:
                                cond.wait(0.01)
                            finished = state["arrived"] and not any(mine) and u.idle
                        if finished:
                            return
                        # only this worker takes from its queues
                        if grouped:
                            u.feed(queues, now())
                        else:
                            u.feed(mine[0], now())
                        u.launch()
                        if not u.in_flight:
                            continue
                        for r in u.poll(wait=True):
                            r._copied.synchronize()
                            r.t_done = now()
            except BaseException as e:  # surface worker failures to the caller
                errors.append(e)

        threads = [threading.Thread(target=worker, args=(u,), daemon=True) for u in self._units()]
        # No garbage collection while the workers run: a collection triggered in one worker runs
        # the finalizers of unreachable library objects there (plan destruction synchronises the
        # device and frees memory), while another worker may be capturing a tick's CUDA graph on its
        # stream. Collect before, and let the collector run again once the workers are joined.
        gc_was_enabled = gc.isenabled()
        gc.collect()
        gc.disable()
        try:
            return self._serve_threads(threads, pending, queues, cond, state, now, realtime, errors)
        finally:
            if gc_was_enabled:
                gc.enable()

    def _serve_threads(self, threads, pending, queues, cond, state, now, realtime, errors) -> float:
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

    def close(self) -> None:
        """Release the groups, then the buckets: each engine (it waits for its stream) before its plan."""
        for g in self.groups:
            g.close()
        self.groups = []
        for b in self.buckets.values():
            b.close()
        self.buckets = {}

    def __enter__(self) -> "SolveServer":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    @property
    def launches(self) -> int:
        return sum(b.launches for b in self.buckets.values()) + sum(g.launches for g in self.groups)

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
