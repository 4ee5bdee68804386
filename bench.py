"""Benchmark: 2D incompressible Navier-Stokes (vorticity form), N = 256^2, batch 64,
1000 SETDRK4 steps of dt = 1e-3, nu = 1e-3, FP32 -- DOF*steps/s.

One bench step = one whole integration of the workload (1000 time steps of the
64-sample batch) from the same seeded initial vorticity (Gaussian random
field, E(k) ~ k^4 exp(-(k/4)^2), zero mean, unit RMS).

  value    : device-resident throughput: the half spectra are in HBM when the
             timed region starts; the fused kernels run through the C ABI.
  e2e      : the same metric through the public API
             (NavierStokesVorticity(1000).integrate) with the initial field in
             pinned host memory and the final field copied back every step.
  roofline : the dominant kernel (the column pass) timed with CUDA events on its
             stream in a separate instrumented pass, algorithmic bytes per launch
             from the kernel's reads and writes; peak = measured HBM copy rate.
  cpu_baseline / --impl reference : the numpy restatement of the reference's
             algorithm (oracle/spectral.py) in complex64 on all host cores, on a
             bounded sample of the same workload.
  torch_gpu_reference / reference_cpu : the reference package itself (installed
             under baseline/_ref) on the same GPU, and on the host cores on a
             bounded sample of the batch.
  accuracy_vs_fp64 : the first samples of our result against the reference's
             own integrator run in float64 on the GPU, after 10, 100 and 1000
             steps, beside the reference's own float32 run of the same samples
             against the same float64 run.

Under torchrun every rank integrates its own batch of 64 (replicas, weak
scaling, no collective on the data path); the time is the max over ranks.
"""

from __future__ import annotations

import argparse
import concurrent.futures as cf
import ctypes
import functools
import json
import math
import os
import statistics
import subprocess
import sys
import time
from typing import Optional

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

N = 256
BATCH = 64
TIME_STEPS = 1000
DT = 1e-3
RE = 1000.0
SEED = 2024
MESH = [(0.0, 2 * math.pi, N), (0.0, 2 * math.pi, N)]
METRIC = "DOF*steps/s (2D NS vorticity 256^2 x 64, SETDRK4, FP32)"
WORKLOAD = "ns2d_vorticity_256x256_b64_1000steps"
FP64_SAMPLES = 4  # samples of the batch integrated again by the reference in float64 (accuracy leg)
ACCURACY_STEPS = (10, 100, 1000)  # step counts at which the accuracy leg compares the results


def _peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def max_over_ranks(value: float, dist, device=None) -> float:
    """Max of a per-rank value over all ranks (the slowest rank's time); identity without dist."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, world: int, ms_max: float) -> float:
    """Whole-job throughput: the units of all ranks over the slowest rank's time (weak scaling)."""
    return world * units_per_rank / (ms_max * 1e-3)


def initial_vorticity(batch: int, seed: int = SEED) -> np.ndarray:
    from torchfsm_gb300 import initial

    return initial.gaussian_random_field((N, N), batch, 1, initial.vorticity_spectrum, seed).astype(np.float32)


# ---------------------------------------------------------------------------
# CPU restatement of the reference (oracle), timed on the host cores
# ---------------------------------------------------------------------------
@functools.lru_cache(maxsize=1)
def _cpu_port_step_setup():
    """The oracle's mesh, nonlinear closure and SETDRK4 tables (complex64) of the headline workload."""
    from oracle import spectral as S

    mesh = S.OMesh(MESH, np.float32)
    nonlinear = S.make_nonlinear(mesh, [(-1.0, "vorticity_convection")])
    lin = S.linear_symbol(mesh, [(1.0 / RE, ("laplacian",))], 1)
    tabs = S.build_tables("setdrk4", lin, DT)
    tabs = {k: (v if k == "dt" else np.asarray(v).astype(mesh.complex_dtype if np.iscomplexobj(v) else mesh.real_dtype))
            for k, v in tabs.items()}
    return mesh, nonlinear, tabs


def cpu_reference_throughput(samples: int, time_steps: int, threads: int) -> dict:
    """The oracle's restatement of the reference's step (numpy complex64) on the host cores: the
    mesh, the nonlinear closure and the SETDRK4 tables are built once, as the reference builds its
    integrator once per (operator, mesh, dt); the timed region is ``time_steps`` steps of each of
    ``samples`` fields, one field per thread."""
    from oracle import spectral as S

    w0 = initial_vorticity(samples, seed=SEED + 1)
    mesh, nonlinear, tabs = _cpu_port_step_setup()
    u_hat = [mesh.fft(w0[i : i + 1].astype(np.float32)) for i in range(samples)]

    def one(i):
        u = u_hat[i]
        for _ in range(time_steps):
            u = S.stage_step("setdrk4", tabs, nonlinear, u)
        return u

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(one, range(samples)))
    elapsed = time.perf_counter() - t0
    dof_steps = samples * N * N * time_steps
    return {"value": dof_steps / elapsed, "unit": "DOF*steps/s", "cores": threads, "kind": "port",
            "sample": f"{samples} samples x {time_steps} SETDRK4 steps of the 256^2 workload "
                      f"(numpy complex64 restatement, {threads} threads; tables built once, outside the timing)",
            "seconds": elapsed}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in getattr(self, "lines", []):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# fused path
# ---------------------------------------------------------------------------
def run_fused(args, rank: int, world: int, dist) -> dict:
    import torch

    import __graft_entry__ as entry

    entry.build()
    from torchfsm_gb300 import pde

    device = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(device)
    B = BATCH
    w0 = initial_vorticity(B, seed=SEED + rank)
    op = pde.NavierStokesVorticity(RE)
    # register + build the plan once (the reference's timing protocol: warm-up call registers the mesh)
    u_dev = torch.tensor(w0, device=device).unsqueeze(1) if w0.ndim == 3 else torch.tensor(w0, device=device)
    op.integrate(u_0=u_dev, mesh=MESH, dt=DT, step=1)
    integ = op._state_dict["integrator"]
    plan, sp = integ.plan, integ.spectral
    state0 = sp.to_half(u_dev).contiguous()
    state = state0.clone()
    ws = torch.empty(plan.workspace_bytes(B, TIME_STEPS), dtype=torch.uint8, device=device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    launches_per_step = plan.launch_count(TIME_STEPS, B)

    def step():
        state.copy_(state0)
        plan.integrate_half(state, TIME_STEPS, workspace=ws)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(device)
    times = []
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(device.index) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)  # evict L2 between timed iterations
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    ms = max_over_ranks(sum(times) / len(times), dist, device)
    finite = bool(torch.isfinite(torch.view_as_real(state)).all().item())

    # e2e through the public API with host buffers
    host_in = torch.tensor(w0).pin_memory()
    host_in = host_in if host_in.dim() == 4 else host_in.unsqueeze(1)
    e2e_times = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        u = host_in.to(device, non_blocking=True)
        out = op.integrate(u_0=u, dt=DT, step=TIME_STEPS)
        out_h = out.cpu()
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_times.append((t1 - t0) * 1e3)
    e2e_ms = max_over_ranks(sum(e2e_times) / len(e2e_times), dist, device)
    # end to end with the build: a fresh operator's first call (mesh registration, FP64 phi tables,
    # plan and workspace) on the same host input, untimed by the steady-state figures above
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fresh = pde.NavierStokesVorticity(RE)
    fresh.integrate(u_0=host_in.to(device, non_blocking=True), mesh=MESH, dt=DT, step=TIME_STEPS).cpu()
    first_ms = max_over_ranks((time.perf_counter() - t0) * 1e3, dist, device)
    del fresh

    # instrumented pass: per-kernel CUDA-event timing of one integration
    prof = profile_kernels(plan, state0, ws, device)

    # the reference's torch GPU path on the same inputs (rank 0 only)
    torch_ref = None
    if rank == 0 and not args.no_torch_reference:
        def ours_after(k):
            return op.integrate(u_0=u_dev, dt=DT, step=k)

        torch_ref = torch_gpu_reference(device, w0, ours_half=ours_after)
    # accuracy: the first samples of the e2e result against the reference's FP64 run of all 1000 steps
    fp64 = None
    if rank == 0 and not args.no_fp64_reference:
        w = w0 if w0.ndim == 4 else w0[:, None]
        ours_by_step = {TIME_STEPS: out_h[:FP64_SAMPLES]}
        for k in ACCURACY_STEPS:
            if k != TIME_STEPS:
                ours_by_step[k] = op.integrate(u_0=u_dev, dt=DT, step=k)[:FP64_SAMPLES].cpu()
        fp64 = accuracy_by_step(lambda R: R.pde.NavierStokesVorticity(RE), MESH, w[:FP64_SAMPLES], DT,
                                ACCURACY_STEPS, ours_by_step, device)
    return {"ms": ms, "e2e_ms": e2e_ms, "finite": finite, "clocks": clk.summary(), "launches": launches_per_step,
            "prof": prof, "h2d": host_in.numel() * 4, "d2h": out_h.numel() * out_h.element_size(),
            "B": B, "torch_ref": torch_ref, "fp64": fp64, "first_ms": first_ms}


def _import_reference():
    """The unmodified reference package installed under baseline/_ref, or (None, reason)."""
    refdir = os.path.join(REPO, "baseline", "_ref")
    if not os.path.isdir(os.path.join(refdir, "torchfsm")):
        return None, "reference not installed under baseline/_ref"
    if refdir not in sys.path:
        sys.path.insert(0, refdir)
    try:
        import torchfsm as R
        import torchfsm.mesh  # noqa: F401
        import torchfsm.pde  # noqa: F401
        import torchfsm.traj_recorder  # noqa: F401
    except Exception as e:  # noqa: BLE001
        return None, f"reference import failed: {type(e).__name__}: {e}"
    return R, None


def reference_steady_step_ms(R, make_op, mesh, u, dt, k1: int, k2: int) -> dict:
    """Steady per-step time of the reference's own integrate on the GPU: the difference of a k2-step
    and a k1-step call (each call carries the reference's fixed gc/empty_cache cost), CUDA events."""
    import torch

    op = make_op(R)
    m = R.mesh.MeshGrid(mesh, device=u.device)
    op.integrate(u_0=u, mesh=m, dt=dt, step=1)  # registers the mesh, builds the coefficients

    def timed(k):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        op.integrate(u_0=u, dt=dt, step=k)
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1)

    t1, t2 = timed(k1), timed(k2)
    return {"ms_per_step": (t2 - t1) / (k2 - k1), "steps_timed": [k1, k2], "call_ms": [t1, t2],
            "kind": "reference torch path (cuFFT + ATen), FP32"}


def torch_gpu_reference(device, w0: np.ndarray, ours_half=None, k1: int = 10, k2: int = 60) -> dict:
    """The reference's own torch path (cuFFT + ATen) on the same GPU, same config and inputs.

    Runs the unmodified reference package installed under baseline/_ref through its public
    API (NavierStokesVorticity(1000).integrate on a cuda MeshGrid, default SETDRK4). Each
    integrate call carries a fixed host cost (gc.collect + empty_cache), so the steady
    per-step time is the difference of a k2-step and a k1-step call, both timed with CUDA
    events. Where our final state after k1 steps is given, the rel-L2 distance of the two
    FP32 results is reported as well."""
    import torch

    R, why = _import_reference()
    if R is None:
        return {"unavailable": why}
    mesh = R.mesh.MeshGrid(MESH, device=device)
    op = R.pde.NavierStokesVorticity(RE)
    u = torch.tensor(w0, device=device)
    u = u if u.dim() == 4 else u.unsqueeze(1)
    torch.cuda.synchronize()
    t_build = time.perf_counter()
    op.integrate(u_0=u, mesh=mesh, dt=DT, step=2)  # registers the mesh, builds the coefficients
    torch.cuda.synchronize()
    build_ms = (time.perf_counter() - t_build) * 1e3

    def timed(k):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record()
        out = op.integrate(u_0=u, dt=DT, step=k)
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1), (time.perf_counter() - t0) * 1e3, out

    t1, w1, out1 = timed(k1)
    t2, w2, _ = timed(k2)
    per_step = (t2 - t1) / (k2 - k1)
    B = u.shape[0]
    res = {"value": B * N * N / (per_step * 1e-3), "unit": "DOF*steps/s", "ms_per_step": per_step,
           "steps_timed": [k1, k2], "call_ms": [t1, t2], "kind": "reference torch path (cuFFT + ATen), FP32",
           "first_call_with_build_ms": build_ms, "first_call_steps": 2,
           "version": getattr(R, "__version__", "0.0.4")}
    if ours_half is not None:
        ours = ours_half(k1)
        res["rel_l2_vs_fused_after_%d_steps" % k1] = float(
            torch.linalg.vector_norm(ours - out1) / torch.linalg.vector_norm(out1))
    return res


def reference_cpu_throughput(samples: int, k1: int = 1, k2: int = 4, threads: int = 0) -> dict:
    """The reference's own path on the host cores: the unmodified package under baseline/_ref,
    ``NavierStokesVorticity(1000).integrate`` on a CPU mesh in float32 (torch CPU FFTs and
    elementwise kernels, all host threads), on a bounded sample of the workload: ``samples`` of
    the 64 seeded fields. Each integrate call carries the reference's fixed gc/empty_cache cost,
    so the steady time per step is the difference of a k2-step and a k1-step call."""
    import torch

    R, why = _import_reference()
    if R is None:
        return {"unavailable": why}
    threads = threads or os.cpu_count() or 1
    prev = torch.get_num_threads()
    torch.set_num_threads(threads)
    try:
        return _reference_cpu_steady(R, samples, k1, k2, threads)
    except Exception as e:  # noqa: BLE001 -- a baseline leg must not cost the throughput line
        return {"unavailable": f"{type(e).__name__}: {e}"}
    finally:
        torch.set_num_threads(prev)


def _reference_cpu_steady(R, samples: int, k1: int, k2: int, threads: int) -> dict:
    import torch

    u = torch.tensor(initial_vorticity(samples, seed=SEED))
    u = u if u.dim() == 4 else u.unsqueeze(1)
    op = R.pde.NavierStokesVorticity(RE)
    op.integrate(u_0=u, mesh=MESH, dt=DT, step=1)  # registers the mesh, builds the coefficients

    def timed(k):
        t0 = time.perf_counter()
        op.integrate(u_0=u, dt=DT, step=k)
        return time.perf_counter() - t0

    t1, t2 = timed(k1), timed(k2)
    per_step = max(t2 - t1, 1e-9) / (k2 - k1)
    return {"value": samples * N * N / per_step, "unit": "DOF*steps/s", "ms_per_step": per_step * 1e3,
            "cores": threads, "kind": "reference package on the host cores (torch CPU), FP32",
            "sample": f"{samples} samples of the 256^2 batch, steady step from a {k2}- and a {k1}-step call",
            "call_s": [t1, t2], "version": getattr(R, "__version__", "0.0.4")}


def fp64_reference_rel_l2(make_op, mesh, u0: np.ndarray, dt: float, steps: int, ours, device) -> dict:
    """Relative L2 distance of a result of ours from the reference's own integrator run in float64.

    The unmodified reference (baseline/_ref) integrates ``u0`` with ``make_op(R).integrate`` in
    float64 on ``device``: its mesh and coefficient tables follow the input's dtype
    (``operator/_base.py:553-559``), so the transforms run in complex128 and the SETDRK4 contour
    coefficients in FP64. ``ours`` is our FP32 result for the same initial field, mesh, dt and
    step count. Any failure is reported as ``unavailable`` and leaves the rest of the line intact."""
    import torch

    R, why = _import_reference()
    if R is None:
        return {"unavailable": why}
    try:
        u = torch.tensor(np.asarray(u0, dtype=np.float64), device=device)
        t0 = time.perf_counter()
        ref = make_op(R).integrate(u_0=u, mesh=mesh, dt=dt, step=steps)
        if ref.device.type == "cuda":
            torch.cuda.synchronize(ref.device)
        wall = time.perf_counter() - t0
        if ref.dtype != torch.float64:
            return {"unavailable": f"reference returned {ref.dtype}, not float64"}
        ours64 = torch.as_tensor(ours).to(device=ref.device, dtype=torch.float64).reshape(ref.shape)
        err = float(torch.linalg.vector_norm(ours64 - ref) / torch.linalg.vector_norm(ref))
        return {"rel_l2": err, "samples": int(u.shape[0]), "steps": steps, "reference_wall_s": wall,
                "kind": f"reference integrate in float64 (complex128 transforms) on {ref.device.type}",
                "version": getattr(R, "__version__", "0.0.4")}
    except Exception as e:  # noqa: BLE001 -- the accuracy leg must not cost the throughput line
        return {"unavailable": f"{type(e).__name__}: {e}"}


def accuracy_by_step(make_op, mesh, u0: np.ndarray, dt: float, checkpoints, ours_by_step: dict, device) -> dict:
    """Relative L2 distance from the reference's own float64 run at several step counts, for our
    FP32 results and for the reference's own FP32 run of the same fields.

    The unmodified reference (baseline/_ref) integrates ``u0`` twice with ``make_op(R).integrate``
    on ``device`` and a recorder that keeps the frames at ``checkpoints``: once in float64 (complex128
    transforms, FP64 contour coefficients: the reference follows the input's dtype,
    ``operator/_base.py:553-559``) and once in float32. ``ours_by_step[k]`` is our result after k
    steps from the same fields. Also reports, at the last checkpoint, the largest relative
    difference of our energy spectrum from the FP64 one over the shells inside the 2/3 rule (the
    comparison a chaotic run keeps). Failures are reported as ``unavailable``."""
    import torch

    R, why = _import_reference()
    if R is None:
        return {"unavailable": why}
    try:
        ks = sorted(int(k) for k in checkpoints)
        wanted = set(ks)

        def run(dtype):
            rec = R.traj_recorder.AutoRecorder(control_func=lambda s: s in wanted)
            u = torch.tensor(np.asarray(u0), dtype=dtype, device=device)
            t0 = time.perf_counter()
            traj = make_op(R).integrate(u_0=u, mesh=mesh, dt=dt, step=ks[-1], trajectory_recorder=rec)
            if traj.device.type == "cuda":
                torch.cuda.synchronize(traj.device)
            return traj, time.perf_counter() - t0

        ref64, wall = run(torch.float64)
        ref32, _ = run(torch.float32)
        if ref64.dtype != torch.float64 or ref64.shape[1] != len(ks):
            return {"unavailable": f"reference trajectory {ref64.dtype} {tuple(ref64.shape)}"}

        def rel(a, b):
            return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))

        ours, theirs = {}, {}
        for i, k in enumerate(ks):
            r = ref64[:, i]
            theirs[str(k)] = rel(ref32[:, i].to(torch.float64), r)
            if k in ours_by_step:
                o = torch.as_tensor(ours_by_step[k]).to(device=r.device, dtype=torch.float64).reshape(r.shape)
                ours[str(k)] = rel(o, r)
        res = {"rel_l2": ours.get(str(ks[-1])), "by_step": ours, "reference_fp32_by_step": theirs,
               "samples": int(ref64.shape[0]), "steps": ks[-1], "reference_wall_s": wall,
               "kind": f"reference integrate in float64 (complex128 transforms) on {ref64.device.type}",
               "version": getattr(R, "__version__", "0.0.4")}
        if ks[-1] in ours_by_step:
            o = torch.as_tensor(ours_by_step[ks[-1]]).to(dtype=torch.float64).reshape(ref64[:, -1].shape)
            e_ours, e_ref = energy_spectrum(o), energy_spectrum(ref64[:, -1])
            kmax = int(2.0 / 3.0 * (min(o.shape[2:]) // 2))
            sel = e_ref[1:kmax + 1]
            res["energy_spectrum_max_rel_diff"] = float(((e_ours[1:kmax + 1] - sel).abs() / sel).max())
        return res
    except Exception as e:  # noqa: BLE001 -- the accuracy leg must not cost the throughput line
        return {"unavailable": f"{type(e).__name__}: {e}"}


def energy_spectrum(u):
    """Energy per integer wavenumber shell of real fields [B, C, n..] (periodic, unit-spaced
    wavenumbers), summed over channels and averaged over the batch: sum over |k| in [s - 1/2,
    s + 1/2) of |u_hat(k)|^2 / (number of points)^2."""
    import torch

    x = u.detach().double().cpu()
    dims = tuple(range(2, x.dim()))
    uh = torch.fft.fftn(x, dim=dims)
    npts = math.prod(x.shape[2:])
    power = (uh.abs() ** 2).sum(1).mean(0) / npts ** 2
    k2 = torch.zeros(x.shape[2:], dtype=torch.float64)
    for i, n in enumerate(x.shape[2:]):
        k = torch.fft.fftfreq(n, d=1.0 / n, dtype=torch.float64)
        shape = [1] * len(dims)
        shape[i] = n
        k2 = k2 + k.reshape(shape) ** 2
    shell = torch.round(torch.sqrt(k2)).long().reshape(-1)
    return torch.zeros(int(shell.max()) + 1, dtype=torch.float64).index_add_(0, shell, power.reshape(-1))


def reference_request_sample(reqs, device, count: int) -> dict:
    """The reference's own ``integrate`` (baseline/_ref, its public API and stock code path) on a
    bounded sample of a serving stream: the ``count`` cheapest requests by DOF*steps, solved one at
    a time on ``device`` (cuda: the reference's torch GPU path; cpu: its CPU path on the host
    cores), each timed from the host field to the host result. Reports DOF*steps/s over the sample
    and, for requests that hold our served result, the largest rel-L2 distance of ours from the
    reference's FP32 result per request kind and the largest relative distance of the two results'
    energy spectra (the comparison that stays meaningful for chaotic KS requests)."""
    import torch

    R, why = _import_reference()
    if R is None:
        return {"unavailable": why}
    try:
        return _reference_request_sample(R, reqs, torch.device(device), count)
    except Exception as e:  # noqa: BLE001 -- a baseline leg must not cost the serving line
        return {"unavailable": f"{type(e).__name__}: {e}"}


def _reference_request_sample(R, reqs, device, count: int) -> dict:
    import torch

    from torchfsm_gb300 import serving

    sample = sorted(reqs, key=lambda r: (r.dof_steps, r.rid))[:count]
    ops, total, secs, diffs, spec_diffs = {}, 0, 0.0, {}, {}
    for r in sample:
        key = (r.kind, r.n)
        if key not in ops:
            ref_op = R.pde.KuramotoSivashinsky() if r.kind == "ks1d" else R.pde.Burgers(serving.BURGERS_NU)
            ops[key] = (ref_op, serving.problem(r.kind, r.n)[1])
        ref_op, mesh = ops[key]
        if device.type == "cuda":
            torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        out = ref_op.integrate(u_0=r.u0.to(device), mesh=mesh, dt=r.dt, step=r.steps).cpu()
        secs += time.perf_counter() - t0
        total += r.dof_steps
        if r.result is not None:
            d = float((r.result.double() - out.double()).norm() / max(float(out.double().norm()), 1e-30))
            diffs[r.kind] = max(diffs.get(r.kind, 0.0), d)
            # chaotic requests (KS over long horizons) are compared by their energy spectra as well
            e_ours, e_ref = energy_spectrum(r.result), energy_spectrum(out)
            ds = float((e_ours - e_ref).norm() / max(float(e_ref.norm()), 1e-30))
            spec_diffs[r.kind] = max(spec_diffs.get(r.kind, 0.0), ds)
    return {"value": total / secs if secs > 0 else None, "unit": "DOF*steps/s", "requests": len(sample),
            "rids": [r.rid for r in sample], "seconds": secs, "device": str(device),
            "cores": torch.get_num_threads() if device.type == "cpu" else None,
            "max_rel_l2_served_vs_reference_fp32": diffs,
            "max_energy_spectrum_rel_diff": spec_diffs,
            "kind": f"reference integrate, one request at a time, on {device.type}"}


def profile_kernels(plan, state0, ws, device) -> dict:
    """Average device time of each kernel kind over one instrumented integration."""
    import torch

    from torchfsm_gb300 import _lib

    lib = _lib.load()
    state = state0.clone()
    ms = (ctypes.c_double * 4)()
    cnt = (ctypes.c_int64 * 4)()
    stream = torch.cuda.current_stream(device).cuda_stream
    steps = 50
    rc = lib.fsm_integrate_profiled(plan.handle, state.shape[0], ctypes.c_void_p(state.data_ptr()), steps,
                                    ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel()),
                                    ctypes.c_void_p(stream), ms, cnt)
    _lib.check(rc)
    torch.cuda.synchronize()
    names = ["column_pass", "row_pass", "prime", "other"]
    return {names[i]: {"launches": int(cnt[i]), "avg_ms": (ms[i] / cnt[i]) if cnt[i] else None}
            for i in range(4)}


# DRAM bytes of one column-pass launch at batch 64, from one ncu capture of `bench.py --ncu-case`
# (dram__bytes_read.sum 35.8 MB + dram__bytes_write.sum 23.2 MB, stage 0 of a SETDRK4 step;
# profiles/ns2d_vorticity_256x256_b64_plane_passes.md).
COLUMN_PASS_DRAM_BYTES = 59.0e6


HK = N // 3 + 1  # last-axis columns of the stage fields kept by the 2/3 rule (stored and read)


def column_pass_bytes(B: int) -> float:
    """Algorithmic bytes of one column-pass launch, averaged over the four SETDRK4 stages.

    Per spectral point (complex64, 8 B): product read 1; state reads (u | u,acc | acc,q | acc)
    and writes (acc,q | acc | acc | u): 11/4; the 4 stage fields written at the HK of H columns
    the 2/3 rule keeps: 4 HK/H. (1 + 2.75 + 2.67) = 6.42 complex accesses at N = 256.
    """
    H = N // 2 + 1
    return (1.0 + 11.0 / 4.0 + 4.0 * HK / H) * 8.0 * B * N * H


def row_pass_bytes(B: int) -> float:
    """The 4 stage fields read at their HK kept columns, 1 product written, per spectral point."""
    H = N // 2 + 1
    return (4.0 * HK / H + 1.0) * 8.0 * B * N * H


def step_model_bytes_per_dof_step() -> float:
    """Both passes of the four SETDRK4 stages per grid point (DOF): 162.6 B at N = 256."""
    H = N // 2 + 1
    return 4.0 * (column_pass_bytes(1) + row_pass_bytes(1)) / (N * N)


# ---------------------------------------------------------------------------
# other workloads (one JSON line each; the default workload is the headline)
# ---------------------------------------------------------------------------
def _pctl(xs, q):
    xs = sorted(xs)
    return xs[min(len(xs) - 1, int(round(q / 100.0 * (len(xs) - 1))))]


# Nominal FP32 FMA rate of a GB300: 152 SMs x 128 FP32 lanes x 2 flop x 2.07 GHz.
FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


def fft_flop_fraction(n: int, channels: int, steps: int, device_ms: float) -> dict:
    """FFT flops of a 1D SETDRK4 solve (per stage one inverse and one forward length-n complex
    transform of the packed real fields, 5 n log2 n flops each, counted as the conventional
    2.5 n log2 n per real transform: 12 real transforms per step, 30 log2 n flops per DOF*step)
    against the nominal FP32 FMA rate."""
    per_dof_step = 30.0 * math.log2(n)
    flops = per_dof_step * n * channels * steps
    achieved = flops / (device_ms * 1e-3) / 1e12
    return {"fft_flops_per_dof_step": per_dof_step, "achieved_tflops": achieved,
            "peak_tflops": FP32_NOMINAL_TFLOPS, "frac": achieved / FP32_NOMINAL_TFLOPS,
            "peak_source": "nominal FP32 FMA rate (152 SMs x 128 lanes x 2 flop x 2.07 GHz)"}


def run_burgers1d(args):
    """1D viscous Burgers, N = 128, nu = 0.01, L = 1, u0 = sin(2 pi x) + 0.5, dt = 0.01, 200 steps,
    batch 1, AutoRecorder (201 frames): solve latency through the public API."""
    import torch

    import __graft_entry__ as entry

    entry.build()
    from oracle import spectral as S
    from torchfsm_gb300 import pde
    from torchfsm_gb300.traj_recorder import AutoRecorder

    n, steps, dt = 128, 200, 0.01
    mesh = [(0.0, 1.0, n)]
    x = np.arange(n) / n
    u0h = torch.tensor((np.sin(2 * np.pi * x) + 0.5).reshape(1, 1, n), dtype=torch.float32).pin_memory()
    op = pde.Burgers(0.01)
    device = torch.device("cuda", 0)
    op.integrate(u_0=u0h.to(device), mesh=mesh, dt=dt, step=1)
    lat = []
    for i in range(args.warmup + max(args.steps, 20)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rec = AutoRecorder()
        traj = op.integrate(u_0=u0h.to(device, non_blocking=True), dt=dt, step=steps, trajectory_recorder=rec)
        out = traj.cpu()
        t1 = time.perf_counter()
        if i >= args.warmup:
            lat.append((t1 - t0) * 1e3)
    # device time of the fused kernel alone (one launch for all 200 steps and the 201 frames)
    integ = op._state_dict["integrator"]
    state0 = integ.spectral.to_half(u0h.to(device))
    traj_h = torch.empty((1, steps + 1, 1, n // 2 + 1), dtype=torch.complex64, device=device)
    ws = torch.empty(integ.plan.workspace_bytes(1, steps), dtype=torch.uint8, device=device)
    dev = []
    for i in range(args.warmup + 20):
        st = state0.clone()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        integ.plan.integrate_half(st, steps, slots=list(range(steps + 1)), traj=traj_h, workspace=ws)
        e1.record()
        e1.synchronize()
        if i >= args.warmup:
            dev.append(e0.elapsed_time(e1))
    u0 = np.sin(2 * np.pi * x).reshape(1, 1, n) + 0.5
    _, ref = S.integrate(u0, mesh, [(0.01, ("laplacian",))], [(-1.0, "convection")], dt, steps, record=lambda i: True)
    err = S.rel_l2(out.numpy(), ref)
    t0 = time.perf_counter()
    reps = 5
    for _ in range(reps):
        S.integrate(u0.astype(np.float32), mesh, [(0.01, ("laplacian",))], [(-1.0, "convection")], dt, steps,
                    record=lambda i: True, real_dtype=np.float32)
    cpu_s = (time.perf_counter() - t0) / reps
    p50 = _pctl(lat, 50)
    # the reference's torch path on the same GPU: the same call (AutoRecorder, host in/out)
    R, why = _import_reference()
    if R is None:
        torch_ref = {"unavailable": why}
    else:
        rop = R.pde.Burgers(0.01)
        rmesh = R.mesh.MeshGrid(mesh, device=device)
        rop.integrate(u_0=u0h.to(device), mesh=rmesh, dt=dt, step=1)
        rl = []
        for i in range(3 + 10):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rtraj = rop.integrate(u_0=u0h.to(device, non_blocking=True), dt=dt, step=steps,
                                  trajectory_recorder=R.traj_recorder.AutoRecorder())
            rtraj.cpu()
            if i >= 3:
                rl.append((time.perf_counter() - t0) * 1e3)
        torch_ref = {"latency_ms": {"p50": _pctl(rl, 50), "p99": _pctl(rl, 99), "n": len(rl)},
                     "value": n * steps / (_pctl(rl, 50) * 1e-3), "unit": "DOF*steps/s",
                     "kind": "reference torch path (cuFFT + ATen), FP32, same call with AutoRecorder",
                     "fused_e2e_over_reference": _pctl(rl, 50) / p50}
    line = {"metric": "DOF*steps/s (1D Burgers N=128, 200 SETDRK4 steps, 201 recorded frames)",
            "value": n * steps / (statistics.median(dev) * 1e-3), "unit": "DOF*steps/s", "n_gpus": 1,
            "steps": len(lat), "warmup": args.warmup, "ms_per_step": statistics.median(dev),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/c64",
            "data": "u0 = sin(2 pi x) + 0.5",
            "config": {"workload": "burgers1d_n128_200steps", "rel_l2_traj_vs_fp64": err},
            "latency_ms": {"p50": p50, "p99": _pctl(lat, 99), "n": len(lat),
                           "what": "Burgers(0.01).integrate with AutoRecorder, pinned host u0 in, trajectory out"},
            "e2e": {"value": n * steps / (p50 * 1e-3), "unit": "DOF*steps/s", "h2d_bytes_per_step": n * 4,
                    "d2h_bytes_per_step": out.numel() * 4},
            "gpu_launches": 1,
            "roofline": {"bound": "latency", "note": "one 128-point line per CTA; all 200 steps in one launch",
                         "device_ms": statistics.median(dev),
                         "fft_flop_fraction": fft_flop_fraction(n, 1, steps, statistics.median(dev))},
            "cpu_baseline": {"value": n * steps / cpu_s, "unit": "DOF*steps/s", "cores": 1, "kind": "port",
                             "sample": "the whole workload, numpy complex64 restatement, 1 thread"},
            "torch_gpu_reference": torch_ref}
    return line


def run_burgers3d(args):
    """3D viscous Burgers (3 channels), 256^3, nu = 0.005, dt = 1e-3, 200 steps, batch 1,
    u0 = GRF with E(k) ~ k^2 exp(-(k/3)^2)."""
    import torch

    import __graft_entry__ as entry

    entry.build()
    from torchfsm_gb300 import initial, pde

    n, steps, dt = 256, 200, 1e-3
    mesh = [(0.0, 2 * math.pi, n)] * 3
    device = torch.device("cuda", 0)
    u0 = torch.tensor(initial.gaussian_random_field((n, n, n), 1, 3, initial.velocity_spectrum, SEED)
                      .astype(np.float32), device=device)
    op = pde.Burgers(0.005)
    op.integrate(u_0=u0, mesh=mesh, dt=dt, step=1)
    integ = op._state_dict["integrator"]
    plan = integ.plan
    state0 = integ.spectral.to_half(u0)
    state = state0.clone()
    ws = torch.empty(plan.workspace_bytes(1, steps), dtype=torch.uint8, device=device)
    for _ in range(args.warmup):
        state.copy_(state0)
        plan.integrate_half(state, steps, workspace=ws)
    torch.cuda.synchronize()
    times = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            state.copy_(state0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            plan.integrate_half(state, steps, workspace=ws)
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    ms = statistics.mean(times)
    dof_steps = 3 * n ** 3 * steps
    prof = profile_kernels(plan, state0, ws, device)
    finite = bool(torch.isfinite(torch.view_as_real(state)).all().item())
    # e2e through the public API: pinned host field in, final field back to the host, every step
    host_in = u0.cpu().pin_memory()
    e2e_times = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out_h = op.integrate(u_0=host_in.to(device, non_blocking=True), dt=dt, step=steps).cpu()
        if i >= args.warmup:
            e2e_times.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = statistics.mean(e2e_times)
    e2e = {"value": dof_steps / (e2e_ms * 1e-3), "unit": "DOF*steps/s", "h2d_bytes_per_step": host_in.numel() * 4,
           "d2h_bytes_per_step": out_h.numel() * out_h.element_size(), "ms_per_step": e2e_ms}
    del out_h
    R, why = _import_reference()
    if R is None:
        torch_ref = {"unavailable": why}
    else:
        del ws
        torch.cuda.empty_cache()
        torch_ref = reference_steady_step_ms(R, lambda R: R.pde.Burgers(0.005), mesh, u0, dt, 1, 4)
        torch_ref["value"] = 3 * n ** 3 / (torch_ref["ms_per_step"] * 1e-3)
        torch_ref["unit"] = "DOF*steps/s"
        torch_ref["fused_device_over_reference"] = (dof_steps / (ms * 1e-3)) / torch_ref["value"]
        torch_ref["peak_mem_gb"] = torch.cuda.max_memory_allocated(device) / 1e9
    # accuracy: our field after 50 steps against the reference's float64 run of the same 50 steps
    fp64 = None
    if not args.no_fp64_reference:
        ours50 = op.integrate(u_0=u0, dt=dt, step=50)
        fp64 = fp64_reference_rel_l2(lambda R: R.pde.Burgers(0.005), mesh, u0.cpu().numpy(), dt, 50, ours50, device)
        del ours50
    line = {"metric": "DOF*steps/s (3D Burgers 256^3 x 3 channels, SETDRK4, FP32)", "value": dof_steps / (ms * 1e-3),
            "unit": "DOF*steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/c64",
            "data": "synthetic (seeded GRF velocity)",
            "config": {"workload": "burgers3d_256cubed_200steps", "result_finite": finite,
                       "l2": "inputs (200 MB state, 1.6 GB workspace) larger than L2",
                       "rel_l2_vs_fp64_after_50_steps": (fp64 or {}).get("rel_l2")},
            "accuracy_vs_fp64": fp64,
            "e2e": e2e,
            "gpu_launches": plan.launch_count(steps, 1) * args.steps,
            "roofline": {"bound": "hbm", "per_kernel_ms": {k: v["avg_ms"] for k, v in prof.items() if v["launches"]},
                         "step_model_bytes_per_dof_step": 276,
                         "step_achieved_gbs": 276.0 * dof_steps / (ms * 1e-3) / 1e9, "peak": _peaks()[0]},
            "torch_gpu_reference": torch_ref,
            "clocks": clk.summary()}
    return line


def run_serving(args):
    """Mixed request stream (KS 1D N=256..4096 / 2D Burgers N=64..256, batch 1-32, steps 100-2000,
    dt 0.01-0.1): the continuous-batching server against the plain drop-in run one solve at a time."""
    import torch

    import __graft_entry__ as entry

    entry.build()
    from torchfsm_gb300 import serving

    device = torch.device("cuda", 0)
    count = args.requests
    reqs = serving.make_stream(count, seed=7, rate_hz=0.0)
    phase, t_phase = {}, time.perf_counter()

    def mark(name):
        nonlocal t_phase
        now = time.perf_counter()
        phase[name] = now - t_phase
        t_phase = now

    server = serving.SolveServer(device, hbm_budget_bytes=16 << 30, chunk=args.chunk, priority=args.priority,
                                 group_lines=bool(args.group_lines), group_planes=bool(args.group_planes))
    server.prepare(sorted({(r.kind, r.n) for r in reqs}))
    # warm-up: a few requests through both paths (kernel attributes, plans of the plain path)
    warm = serving.make_stream(8, seed=99, rate_hz=0.0, max_steps=120)
    server.run(warm, realtime=False)
    ops = {}
    for r in warm:
        serving.solve_alone(r, device, ops)
    total = sum(r.dof_steps for r in reqs)
    run = server.run_threaded if args.threaded else server.run
    mark("setup_and_warmup")
    # burst: every request waiting at t = 0
    wall = run(reqs, realtime=False)
    mark("burst")
    serve_tp = total / wall
    burst_lat = [r.t_done - r.arrival for r in reqs]
    # the plain drop-in, one solve at a time, same requests in the same order
    alone_t, max_err, nonfinite_plain = [], 0.0, []
    for r in reqs:
        res, t = serving.solve_alone(r, device, ops)
        alone_t.append(t)
        if not bool(torch.isfinite(res).all()):
            nonfinite_plain.append(r.rid)
            continue
        ref = res.double()
        max_err = max(max_err, float((r.result.double() - ref).norm() / max(ref.norm(), 1e-30)))
    nonfinite_serve = [r.rid for r in reqs if r.finite is False]
    mark("plain")
    # the reference's own path on bounded samples of the same stream (cheapest requests first),
    # beside our one-at-a-time path on the same requests
    alone_by_rid = {r.rid: t for r, t in zip(reqs, alone_t)}
    reference_sample = {}
    for leg, dev, cnt in (("torch_gpu", device, args.ref_requests), ("cpu", "cpu", args.ref_cpu_requests)):
        res = reference_request_sample(reqs, dev, cnt)
        if "rids" in res:
            ours_s = sum(alone_by_rid[i] for i in res["rids"])
            dof = sum(r.dof_steps for r in reqs if r.rid in set(res["rids"]))
            res["plain_value_same_requests"] = dof / ours_s if ours_s > 0 else None
        reference_sample[leg] = res
    plain_tp = total / sum(alone_t)
    mark("reference_samples")
    # Poisson arrivals at rates below the server's measured capacity: latency of each request
    # against its own one-at-a-time time (the streams hold the same requests at every rate)
    sweep = []
    loads = sorted({float(x) for x in str(args.loads).split(",") if x} | {args.load})
    for load in loads:
        rq = serving.make_stream(count, seed=7, rate_hz=load * count / wall)
        w = run(rq, realtime=True)
        lt = [r.t_done - r.arrival for r in rq]
        rt = [l / a for l, a in zip(lt, alone_t)]
        sweep.append({"load": load, "rate_hz": load * count / wall, "wall_s": w,
                      "latency_s": {"p50": _pctl(lt, 50), "p99": _pctl(lt, 99)},
                      "latency_over_isolated": {"p50": _pctl(rt, 50), "p99": _pctl(rt, 99)},
                      "p99_over_isolated_p99": _pctl(lt, 99) / _pctl(alone_t, 99)})
        if load == args.load:
            rate, wall2, lat, ratio = load * count / wall, w, lt, rt
    mark("poisson_sweep")
    line = {"metric": "DOF*steps/s of a mixed solve stream (continuous batching vs one solve at a time)",
            "value": serve_tp, "unit": "DOF*steps/s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": wall * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32/c64", "data": "synthetic (seeded band-limited fields)",
            "config": {"workload": f"serving_{count}_requests", "chunk_steps": args.chunk,
                       "host_loop": "thread per bucket" if args.threaded else "single loop",
                       "high_priority_buckets": args.priority,
                       "cuda_graphs": f"replayed per (slots, steps) shape for ticks of <= {serving.GRAPH_MAX_STEPS} steps",
                       "mix": "KS 1D L=32pi N in {256..4096} | 2D Burgers nu=0.01 N in {64,128,256}; batch 1-32; "
                              "steps 100-2000; dt 0.01-0.1; ICs |k|<=8, RMS 1 (KS) / 0.25 (Burgers)"},
            "serving": {"throughput_serve": serve_tp, "throughput_plain": plain_tp,
                        "speedup_vs_plain": serve_tp / plain_tp,
                        "burst_latency_s": {"p50": _pctl(burst_lat, 50), "p99": _pctl(burst_lat, 99)},
                        "poisson_rate_hz": rate, "poisson_wall_s": wall2,
                        "latency_s": {"p50": _pctl(lat, 50), "p99": _pctl(lat, 99)},
                        "isolated_latency_s": {"p50": _pctl(alone_t, 50), "p99": _pctl(alone_t, 99)},
                        "latency_over_isolated": {"p50": _pctl(ratio, 50), "p99": _pctl(ratio, 99)},
                        "poisson_sweep": sweep, "graph_replays": server.graph_replays, "phase_seconds": phase,
                        "line_groups": [[b.n for b in g.buckets] for g in server.groups],
                        "target": "throughput >= 3x the plain path (burst); p99 latency <= 2x the isolated p99 "
                                  "(same requests one at a time) at a stated Poisson load",
                        "loads_meeting_p99_target": [x["load"] for x in sweep if x["p99_over_isolated_p99"] <= 2.0],
                        "max_rel_diff_mix_vs_alone": max_err,
                        "nonfinite_requests": {"serve": len(nonfinite_serve), "plain": len(nonfinite_plain),
                                               "same_requests": nonfinite_serve == nonfinite_plain},
                        "reference_sample": reference_sample},
            "gpu_launches": server.launches,
            "e2e": {"value": serve_tp, "unit": "DOF*steps/s",
                    "h2d_bytes_per_step": sum(r.u0.numel() * 4 for r in reqs),
                    "d2h_bytes_per_step": sum(r.u0.numel() * 4 for r in reqs)}}
    server.close()
    return line


def run_burgers2d_grad(args):
    """Differentiable 2D Burgers nu = 0.01, 128^2, batch 16, 500 SETDRK4 steps of dt = 0.005, band-limited
    ICs (|k| <= 6, unit RMS); loss = MSE to the nu = 0.02 run; gradients w.r.t. u0 and nu with checkpoints
    every 50 steps (hand-written adjoint)."""
    import torch

    import __graft_entry__ as entry

    entry.build()
    from torchfsm_gb300 import initial, pde
    from torchfsm_gb300.operator import Convection, Laplacian

    n, B, steps, dt = 128, 16, 500, 0.005
    mesh = [(0.0, 2 * math.pi, n)] * 2
    dev = torch.device("cuda", 0)
    u0h = torch.tensor(initial.band_limited((n, n), B, 2, 6, SEED, 1.0).astype(np.float32))
    u0d = u0h.to(dev)
    with torch.no_grad():
        target = pde.Burgers(0.02).integrate(u_0=u0d, mesh=mesh, dt=dt, step=steps)
    nu = torch.tensor(0.01, device=dev, requires_grad=True)
    op = nu * Laplacian() - Convection()
    with torch.no_grad():
        op.integrate(u_0=u0d, mesh=mesh, dt=dt, step=1)

    def fwd_bwd():
        nu.grad = None
        u = u0d.clone().requires_grad_(True)
        out = op.integrate(u_0=u, dt=dt, step=steps)
        loss = ((out - target) ** 2).mean()
        # the operator's coefficient is the non-leaf tensor 1 * nu, shared by every call
        loss.backward(retain_graph=True)
        return loss.item(), u.grad, nu.grad.item()

    for _ in range(max(1, args.warmup)):
        fwd_bwd()
    times = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loss, gu, gnu = fwd_bwd()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    # forward alone
    ftimes = []
    with torch.no_grad():
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            op.integrate(u_0=u0d, dt=dt, step=steps)
            torch.cuda.synchronize()
            ftimes.append(time.perf_counter() - t0)
    # FP32 central differences in nu through the fused forward; eps = 1e-3 is 10% of nu, so its
    # O(eps^2) error is removed by Richardson extrapolation with eps / 2
    def central(eps):
        with torch.no_grad():
            lp = ((pde.Burgers(0.01 + eps).integrate(u_0=u0d, mesh=mesh, dt=dt, step=steps) - target) ** 2).mean()
            lm = ((pde.Burgers(0.01 - eps).integrate(u_0=u0d, mesh=mesh, dt=dt, step=steps) - target) ** 2).mean()
        return (lp.item() - lm.item()) / (2 * eps)

    fd1, fd2 = central(1e-3), central(5e-4)
    fd = (4 * fd2 - fd1) / 3
    ref = reference_autograd_burgers2d(dev, u0h, target, mesh, dt, steps)
    if "grad_u0" in ref:
        ref["rel_l2_grad_u0_vs_adjoint"] = float(torch.linalg.vector_norm(ref.pop("grad_u0") - gu.double())
                                                 / torch.linalg.vector_norm(gu.double()))
        ref["rel_diff_grad_nu_vs_adjoint"] = abs(ref["grad_nu"] - gnu) / abs(ref["grad_nu"])
    dof_steps = B * 2 * n * n * steps
    tb = statistics.median(times)
    tf = statistics.median(ftimes)
    line = {"metric": "DOF*steps/s of forward + backward (2D Burgers 128^2 x 16, 500 steps, grads w.r.t. u0 and nu)",
            "value": dof_steps / tb, "unit": "DOF*steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tb * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32/c64", "data": "synthetic (seeded band-limited fields)",
            "config": {"workload": "burgers2d_grad_128x128_b16_500steps", "checkpoint_every": 50},
            "forward_only": {"value": dof_steps / tf, "ms": tf * 1e3},
            "backward_over_forward": tb / tf,
            "gradients": {"loss": loss, "grad_nu_adjoint": gnu, "grad_nu_fd_fp32_eps1e-3": fd1,
                          "grad_nu_fd_fp32_eps5e-4": fd2, "grad_nu_fd_richardson": fd,
                          "rel_diff_vs_richardson": abs(gnu - fd) / abs(fd),
                          "grad_u0_finite": bool(torch.isfinite(gu).all())},
            "reference_autograd": ref}
    return line


def reference_autograd_burgers2d(device, u0h, target, mesh, dt, steps) -> dict:
    """The reference's own autograd gradient on the same GPU and inputs (FP32): nu * Laplacian() -
    Convection() integrated by the unmodified reference installed under baseline/_ref, loss = MSE to
    the same target, d loss / d u0 and d loss / d nu by loss.backward(); timed once."""
    import torch

    R, why = _import_reference()
    if R is None:
        return {"unavailable": why}
    m = R.mesh.MeshGrid(mesh, device=device)
    nu = torch.tensor(0.01, device=device, requires_grad=True)
    op = nu * R.operator.Laplacian() - R.operator.Convection()
    # registers the mesh and builds the coefficients (with grad enabled, so that they depend on nu;
    # no backward here, so their graph is still there for the timed backward)
    op.integrate(u_0=u0h.to(device), mesh=m, dt=dt, step=1)
    x = u0h.to(device).clone().requires_grad_(True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = op.integrate(u_0=x, dt=dt, step=steps)
    loss = ((out - target) ** 2).mean()
    loss.backward()
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    res = {"kind": "reference torch autograd (cuFFT + ATen), FP32", "seconds_fwd_bwd": t,
           "loss": loss.item(), "grad_nu": nu.grad.item(), "grad_u0": x.grad.detach().double(),
           "peak_mem_gb": torch.cuda.max_memory_allocated(device) / 1e9}
    del out, loss, op, x
    torch.cuda.empty_cache()
    return res


def ncu_case(workload: str = "ns2d", n3d: int = 256):
    """Small profiling runs. ns2d: full batch (inputs larger than L2): a 1-step integrate (plan build,
    split launches), then 3 SETDRK4 steps of the whole batch as one launch sequence. burgers3d: n3d^3 x 3 (256 by default; 128 for captures of several
    metrics, whose passes save and restore device memory), 1 warm-up step then 2 steps."""
    import torch

    import __graft_entry__ as entry

    entry.build()
    from torchfsm_gb300 import initial, pde

    if workload == "burgers2d_grad":
        # the differentiable workload's shapes (128^2 x 16, 2 channels), 10 steps, forward + backward
        from torchfsm_gb300.operator import Convection, Laplacian

        device = torch.device("cuda", 0)
        u0 = torch.tensor(initial.band_limited((128, 128), 16, 2, 6, SEED, 1.0).astype(np.float32), device=device)
        nu = torch.tensor(0.01, device=device, requires_grad=True)
        op = nu * Laplacian() - Convection()
        u = u0.clone().requires_grad_(True)
        out = op.integrate(u_0=u, mesh=[(0.0, 2 * math.pi, 128)] * 2, dt=0.005, step=10)
        (out ** 2).mean().backward()
        torch.cuda.synchronize()
        print("ncu case done", bool(torch.isfinite(u.grad).all().item()))
        return
    if workload == "serving":
        # the serving groups' kernels: KS 1D at 256, 1024 and 4096 points advanced by one line launch
        # per tick (k_line_multi), 2D Burgers at 64^2, 128^2 and 256^2 by one launch per pass
        # (k_axis0_multi2, k_plane_row_multi); 8 requests per size, 16 slots per engine, ticks of 8 steps
        from torchfsm_gb300 import _lib, _native, serving
        from torchfsm_gb300.mesh import FourierMesh

        device = torch.device("cuda", 0)
        groups, keep = [], []
        for kind, sizes in (("ks1d", (256, 1024, 4096)), ("burgers2d", (64, 128, 256))):
            stream = torch.cuda.Stream(device)
            pools = []
            for n in sizes:
                op, mesh, C = serving.problem(kind, n)
                f_mesh = FourierMesh(mesh, device=device, dtype=torch.float32)
                op.register_mesh(f_mesh, C)
                prog = _native.lower(op._linear_terms, op._nonlinear_funcs, f_mesh, C, op._de_aliasing_rate)
                with torch.cuda.stream(stream):
                    plan = _native.NativePlan(prog, 0.05, _lib.FSM_SETDRK4, device,
                                              linear_coef64=op._linear_coef64(device), table_batch=16)
                torch.cuda.synchronize()
                pool = _native.ServePool(plan, 16, 8, stream)
                shape = (n,) if kind == "ks1d" else (n, n)
                for rid in range(8):
                    u = initial.band_limited(shape, 2, C, 8, SEED + rid, 1.0 if kind == "ks1d" else 0.25)
                    h = _native.Spectral(plan).to_half(torch.tensor(u, dtype=torch.float32, device=device)).contiguous()
                    pool.submit(rid, 32, 0.02, h)
                    keep.append(h)
                pools.append(pool)
            groups.append((_native.ServeGroup(pools, tick_ms=0.0), pools))
        torch.cuda.synchronize()
        for group, pools in groups:
            for _ in range(4):
                group.tick()
                group.poll(wait=True)
                for p in pools:
                    p.poll(False)
        torch.cuda.synchronize()
        print("ncu case done", all(bool(torch.isfinite(torch.view_as_real(h)).all()) for h in keep))
        for group, pools in groups:
            group.close()
        return
    if workload in ("burgers1d", "ks1d", "heat2d"):
        # the kernels outside the plane and volume passes, on small cases of their workloads:
        # burgers1d: the 1D line kernel at N = 128 (200 steps, 201 frames), the FP64 coefficient kernel
        # and the last-axis transforms; ks1d: the line kernel at N = 4096 (batch 32, 100 steps) and the
        # KS batch-mean kernels (KuramotoSivashinskyHighDim in 1D, N = 1024, batch 8, 50 steps); heat2d:
        # the pointwise kernel of a linear program and the 2D transforms at 256^2 x 64
        from torchfsm_gb300.operator import Laplacian
        from torchfsm_gb300.traj_recorder import AutoRecorder

        device = torch.device("cuda", 0)
        if workload == "burgers1d":
            x = np.arange(128) / 128
            u = torch.tensor((np.sin(2 * np.pi * x) + 0.5).reshape(1, 1, 128), dtype=torch.float32, device=device)
            out = pde.Burgers(0.01).integrate(u_0=u, mesh=[(0.0, 1.0, 128)], dt=0.01, step=200,
                                              trajectory_recorder=AutoRecorder())
        elif workload == "ks1d":
            L = 32 * math.pi
            u = torch.tensor(initial.band_limited((4096,), 32, 1, 8, SEED, 1.0).astype(np.float32), device=device)
            out = pde.KuramotoSivashinsky().integrate(u_0=u, mesh=[(0.0, L, 4096)], dt=0.02, step=100)
            v = torch.tensor(initial.band_limited((1024,), 8, 1, 8, SEED, 0.7).astype(np.float32), device=device)
            out2 = pde.KuramotoSivashinskyHighDim().integrate(u_0=v, mesh=[(0.0, 10 * math.pi, 1024)], dt=0.02,
                                                              step=50)
            out = torch.cat([out.flatten(), out2.flatten()])
        else:
            u = torch.tensor(initial_vorticity(BATCH), device=device)
            out = (0.05 * Laplacian()).integrate(u_0=u, mesh=MESH, dt=1e-3, step=100)
        torch.cuda.synchronize()
        print("ncu case done", bool(torch.isfinite(out).all().item()))
        return
    if workload == "burgers3d":
        n = n3d
        device = torch.device("cuda", 0)
        u0 = torch.tensor(initial.gaussian_random_field((n, n, n), 1, 3, initial.velocity_spectrum, SEED)
                          .astype(np.float32), device=device)
        op = pde.Burgers(0.005)
        op.integrate(u_0=u0, mesh=[(0.0, 2 * math.pi, n)] * 3, dt=1e-3, step=1)
        out = op.integrate(u_0=u0, dt=1e-3, step=2)
        torch.cuda.synchronize()
        print("ncu case done", bool(torch.isfinite(out).all().item()))
        return

    device = torch.device("cuda", 0)
    u = torch.tensor(initial_vorticity(BATCH), device=device)
    op = pde.NavierStokesVorticity(RE)
    op.integrate(u_0=u, mesh=MESH, dt=DT, step=1)
    integ = op._state_dict["integrator"]
    plan = integ.plan
    state = integ.spectral.to_half(u).contiguous()
    ws = torch.empty(plan.workspace_bytes(BATCH, 3), dtype=torch.uint8, device=device)
    # 3 steps of the full batch as one launch sequence (the kernel time of the timed run's parts in
    # one launch each): column passes 0 (priming), 1-4, 5-8, 9-12; row passes 0-3, 4-7, 8-11
    from torchfsm_gb300 import _lib

    ms = (ctypes.c_double * 4)()
    cnt = (ctypes.c_int64 * 4)()
    _lib.check(_lib.load().fsm_integrate_profiled(
        plan.handle, BATCH, ctypes.c_void_p(state.data_ptr()), 3, ctypes.c_void_p(ws.data_ptr()),
        ctypes.c_size_t(ws.numel()), ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream), ms, cnt))
    torch.cuda.synchronize()
    print("ncu case done", bool(torch.isfinite(torch.view_as_real(state)).all().item()))


def _summary(line: dict, keys) -> dict:
    out = {}
    for k in keys:
        cur, src = line, k.split(".")
        for part in src:
            cur = cur.get(part) if isinstance(cur, dict) else None
        out[k] = cur
    return out


def other_workloads(args) -> dict:
    """The other named workloads, run after the headline's timed region and summarised on its line:
    1D Burgers N=128 solve latency, 3D Burgers 256^3 throughput with its FP64 error after 50 steps,
    the differentiable 2D Burgers forward + backward with its gradient checks, and the serving
    stream (burst throughput against the plain path, latency at one Poisson load). Each runs with few
    repetitions (its own workload line, ``--workload``, has the full figures); a failure is reported
    and leaves the headline intact."""
    import argparse as _ap

    small = _ap.Namespace(**dict(vars(args), steps=3, warmup=1))
    legs = {
        "burgers1d_n128_200steps": (run_burgers1d, ["value", "unit", "latency_ms", "config.rel_l2_traj_vs_fp64",
                                                    "torch_gpu_reference.latency_ms",
                                                    "torch_gpu_reference.fused_e2e_over_reference"]),
        "burgers3d_256cubed_200steps": (run_burgers3d, ["value", "unit", "ms_per_step", "e2e.value",
                                                        "config.rel_l2_vs_fp64_after_50_steps",
                                                        "roofline.step_achieved_gbs", "roofline.per_kernel_ms",
                                                        "torch_gpu_reference.value",
                                                        "torch_gpu_reference.fused_device_over_reference"]),
        "burgers2d_grad_128x128_b16_500steps": (run_burgers2d_grad, ["value", "unit", "ms_per_step", "forward_only",
                                                                     "gradients.grad_nu_adjoint",
                                                                     "gradients.rel_diff_vs_richardson",
                                                                     "reference_autograd.seconds_fwd_bwd",
                                                                     "reference_autograd.rel_l2_grad_u0_vs_adjoint",
                                                                     "reference_autograd.rel_diff_grad_nu_vs_adjoint"]),
    }
    serve = _ap.Namespace(**dict(vars(args), requests=args.serve_summary_requests, loads=args.loads,
                                 ref_requests=0, ref_cpu_requests=0))
    if args.serve_summary_requests > 0:
        legs[f"serving_{args.serve_summary_requests}_requests"] = (
            lambda _a: run_serving(serve),
            ["value", "unit", "config.workload", "serving.throughput_plain", "serving.speedup_vs_plain",
             "serving.poisson_rate_hz", "serving.latency_s", "serving.isolated_latency_s",
             "serving.latency_over_isolated", "serving.poisson_sweep", "serving.loads_meeting_p99_target",
             "serving.max_rel_diff_mix_vs_alone", "serving.nonfinite_requests", "serving.line_groups",
             "serving.phase_seconds", "gpu_launches"])
    out = {}
    for name, (fn, keys) in legs.items():
        t0 = time.perf_counter()
        try:
            out[name] = _summary(fn(small), keys)
        except Exception as e:  # noqa: BLE001 -- a summary leg must not cost the headline line
            out[name] = {"unavailable": f"{type(e).__name__}: {e}"}
        out[name]["wall_s"] = time.perf_counter() - t0
    return out


def fused_line(res: dict, args, world: int, cpu: Optional[dict], ref_cpu: Optional[dict]) -> dict:
    """The JSON line of the fused arm from ``run_fused``'s measurements and the CPU baselines."""
    dof_steps = res["B"] * N * N * TIME_STEPS
    value = job_throughput(dof_steps, world, res["ms"])
    e2e_value = job_throughput(dof_steps, world, res["e2e_ms"])
    peak, peak_kind = _peaks()
    col = res["prof"]["column_pass"]
    achieved = column_pass_bytes(res["B"]) / (col["avg_ms"] * 1e-3) / 1e9 if col["avg_ms"] else None
    line = {
        "metric": METRIC, "value": value, "unit": "DOF*steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/c64", "data": "synthetic (seeded GRF vorticity)",
        "config": {"workload": WORKLOAD, "grid": [N, N], "batch_per_gpu": res["B"], "time_steps": TIME_STEPS,
                   "dt": DT, "nu": 1.0 / RE, "integrator": "SETDRK4 (M=16, r=1)",
                   "parallelism": f"replicas x{world}", "l2": "flushed (256 MB write) between timed steps",
                   "result_finite": res["finite"],
                   "rel_l2_vs_fp64": (res["fp64"] or {}).get("rel_l2")},
        "accuracy_vs_fp64": res["fp64"],
        "e2e": {"value": e2e_value, "unit": "DOF*steps/s", "h2d_bytes_per_step": res["h2d"],
                "d2h_bytes_per_step": res["d2h"], "ms_per_step": res["e2e_ms"],
                "first_call_with_build_ms": res["first_ms"]},
        "gpu_launches": res["launches"] * args.steps,
        "roofline": {"bound": "hbm", "kernel": "k_axis0_r2<256, VORTICITY, 2> (column pass, SETDRK4 stages)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": COLUMN_PASS_DRAM_BYTES,
                     "traffic_note": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one stage-0 column pass "
                                     "launch of this workload (bench.py --ncu-case; "
                                     "profiles/ns2d_vorticity_256x256_b64_plane_passes.md)",
                     "peak_source": f"{peak_kind} hbm_gbs",
                     "per_kernel_ms": {k: v["avg_ms"] for k, v in res["prof"].items() if v["launches"]},
                     "step_model_bytes_per_dof_step": step_model_bytes_per_dof_step(),
                     "step_achieved_gbs": step_model_bytes_per_dof_step() * dof_steps / (res["ms"] * 1e-3) / 1e9},
        "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")} if cpu else None,
        "torch_gpu_reference": res["torch_ref"],
        "reference_cpu": ref_cpu,
        "clocks": res["clocks"],
    }
    tr = res["torch_ref"]
    if tr and "value" in tr:
        tr["fused_device_over_reference"] = value / tr["value"]
        tr["fused_e2e_over_reference"] = e2e_value / tr["value"]
    if ref_cpu and "value" in ref_cpu:
        ref_cpu["fused_e2e_over_reference_cpu"] = e2e_value / ref_cpu["value"]
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="fused", choices=["fused", "reference"])
    ap.add_argument("--cpu-samples", type=int, default=16)
    ap.add_argument("--cpu-time-steps", type=int, default=5)
    ap.add_argument("--no-torch-reference", action="store_true",
                    help="skip the reference torch GPU path leg of the ns2d workload")
    ap.add_argument("--ref-cpu-samples", type=int, default=8,
                    help="ns2d: samples of the batch run by the reference package on the host cores (0: skip)")
    ap.add_argument("--no-other-workloads", action="store_true",
                    help="ns2d: skip the summaries of the 1D, 3D and gradient workloads run after the timed region")
    ap.add_argument("--no-fp64-reference", action="store_true",
                    help="skip the accuracy leg (the reference's float64 run of the first samples)")
    ap.add_argument("--requests", type=int, default=2000, help="serving: number of requests")
    ap.add_argument("--loads", default="0.25,0.35",
                    help="serving: Poisson rates measured, as fractions of the burst capacity")
    ap.add_argument("--chunk", type=int, default=50, help="serving: steps per tick")
    ap.add_argument("--ref-requests", type=int, default=20,
                    help="serving: requests of the stream run by the reference's torch GPU path")
    ap.add_argument("--ref-cpu-requests", type=int, default=3,
                    help="serving: requests of the stream run by the reference's CPU path")
    ap.add_argument("--load", type=float, default=0.25, help="serving: the Poisson rate whose figures head the line, as a fraction of capacity")
    ap.add_argument("--threaded", type=int, default=1, help="serving: one host worker thread per bucket")
    ap.add_argument("--serve-summary-requests", type=int, default=2000,
                    help="ns2d: requests of the serving stream summarised on the headline line after its timed "
                         "region (burst, plain path, the --loads Poisson rates; 0: skip)")
    ap.add_argument("--group-lines", type=int, default=1,
                    help="serving: the 1D KS buckets of every size advance together, one launch per tick")
    ap.add_argument("--group-planes", type=int, default=0,
                    help="serving: the 2D Burgers buckets of every size advance together, one launch per pass")
    ap.add_argument("--priority", default="costly", choices=["cheap", "costly"],
                    help="serving: buckets on the high-priority streams")
    ap.add_argument("--workload", default="ns2d",
                    choices=["ns2d", "burgers1d", "burgers3d", "serving", "burgers2d_grad", "ks1d", "heat2d"],
                    help="ns2d: the headline (2D NS vorticity 256^2 x 64); burgers1d: 1D Burgers N=128 latency; "
                         "burgers3d: 3D Burgers 256^3; ks1d, heat2d: --ncu-case only")
    ap.add_argument("--ncu-case", action="store_true",
                    help="small profiling case: one warm-up step, then 3 time steps of the full batch")
    ap.add_argument("--ncu-n", type=int, default=256, help="grid size of the burgers3d profiling case")
    args = ap.parse_args()
    if args.ncu_case:
        ncu_case(args.workload, args.ncu_n)
        return
    if args.workload in ("ks1d", "heat2d"):
        ap.error(f"--workload {args.workload} is a profiling case: use it with --ncu-case")
    if args.workload == "burgers1d" and args.impl == "fused":
        print(json.dumps(run_burgers1d(args)))
        return
    if args.workload == "burgers3d" and args.impl == "fused":
        print(json.dumps(run_burgers3d(args)))
        return
    if args.workload == "serving" and args.impl == "fused":
        print(json.dumps(run_serving(args)))
        return
    if args.workload == "burgers2d_grad" and args.impl == "fused":
        print(json.dumps(run_burgers2d_grad(args)))
        return
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        vals = []
        for i in range(args.warmup + args.steps):
            r = cpu_reference_throughput(min(BATCH, max(threads, args.cpu_samples)), args.cpu_time_steps, threads)
            if i >= args.warmup:
                vals.append(r)
        value = statistics.mean(v["value"] for v in vals)
        r = vals[-1]
        sec = statistics.mean(v["seconds"] for v in vals)
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "DOF*steps/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
                "config": {"workload": WORKLOAD, "grid": [N, N], "batch": BATCH, "time_steps": TIME_STEPS,
                           "dt": DT, "nu": 1.0 / RE, "integrator": "SETDRK4", "sample": r["sample"],
                           "l2": "n/a (host)"},
                "cpu_baseline": dict({k: r[k] for k in ("unit", "cores", "kind", "sample")}, value=value),
                "e2e": {"value": value, "unit": "DOF*steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    dist = None
    if world > 1:
        import torch.distributed as td

        td.init_process_group("nccl")
        dist = td
    res = run_fused(args, rank, world, dist)
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    # the CPU baselines are timed at N = 1 only (the host cores are shared by all ranks otherwise)
    cpu = cpu_reference_throughput(min(BATCH, max(os.cpu_count() or 1, args.cpu_samples)), args.cpu_time_steps,
                                   os.cpu_count() or 1) if world == 1 else None
    ref_cpu = reference_cpu_throughput(args.ref_cpu_samples) if world == 1 and args.ref_cpu_samples > 0 else None
    line = fused_line(res, args, world, cpu, ref_cpu)
    if world == 1 and not args.no_other_workloads:
        line["other_workloads"] = other_workloads(args)
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
