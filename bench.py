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

Under torchrun every rank integrates its own batch of 64 (replicas, weak
scaling, no collective on the data path); the time is the max over ranks.
"""

from __future__ import annotations

import argparse
import concurrent.futures as cf
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import time

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


def _peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def initial_vorticity(batch: int, seed: int = SEED) -> np.ndarray:
    from torchfsm_gb300 import initial

    return initial.gaussian_random_field((N, N), batch, 1, initial.vorticity_spectrum, seed).astype(np.float32)


# ---------------------------------------------------------------------------
# CPU restatement of the reference (oracle), timed on the host cores
# ---------------------------------------------------------------------------
def cpu_reference_throughput(samples: int, time_steps: int, threads: int) -> dict:
    from oracle import spectral as S

    w0 = initial_vorticity(samples, seed=SEED + 1)

    def one(i):
        S.integrate(w0[i : i + 1], MESH, [(1.0 / RE, ("laplacian",))], [(-1.0, "vorticity_convection")], DT,
                    time_steps, real_dtype=np.float32)

    # coefficient build outside the timed region, as for the GPU path
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(one, range(samples)))
    t1 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda i: None, range(samples)))
    elapsed = t1 - t0
    dof_steps = samples * N * N * time_steps
    return {"value": dof_steps / elapsed, "unit": "DOF*steps/s", "cores": threads, "kind": "port",
            "sample": f"{samples} samples x {time_steps} SETDRK4 steps of the 256^2 workload "
                      f"(numpy complex64 restatement, {threads} threads, coefficient build included)",
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
    from torchfsm_gb300 import _lib, _native, pde
    from torchfsm_gb300.mesh import FourierMesh

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
    launches_per_step = plan.launch_count(TIME_STEPS)

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
    ms = sum(times) / len(times)
    if dist is not None:
        t = torch.tensor([ms], device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
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
    e2e_ms = sum(e2e_times) / len(e2e_times)
    if dist is not None:
        t = torch.tensor([e2e_ms], device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())

    # instrumented pass: per-kernel CUDA-event timing of one integration
    prof = profile_kernels(plan, state0, ws, device)
    return {"ms": ms, "e2e_ms": e2e_ms, "finite": finite, "clocks": clk.summary(), "launches": launches_per_step,
            "prof": prof, "h2d": host_in.numel() * 4, "d2h": out_h.numel() * out_h.element_size(),
            "B": B}


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


def column_pass_bytes(B: int) -> float:
    """Algorithmic bytes of one column-pass launch, averaged over the four SETDRK4 stages.

    Per spectral point (complex64, 8 B): product read 1; state reads
    (u | u,acc | acc,q | acc) and writes (acc,q | acc | acc | u); 4 mid fields
    written: (2+6 + 3+5 + 3+5 + 2+5)/4 = 7.75 complex accesses.
    """
    H = N // 2 + 1
    return 7.75 * 8.0 * B * N * H


def row_pass_bytes(B: int) -> float:
    """4 mid fields read + 1 product written per spectral point."""
    H = N // 2 + 1
    return 5.0 * 8.0 * B * N * H


def ncu_case():
    """Full batch (inputs larger than L2), 3 SETDRK4 steps: 25 launches after a 9-launch warm-up."""
    import torch

    import __graft_entry__ as entry

    entry.build()
    from torchfsm_gb300 import pde

    device = torch.device("cuda", 0)
    u = torch.tensor(initial_vorticity(BATCH), device=device)
    op = pde.NavierStokesVorticity(RE)
    op.integrate(u_0=u, mesh=MESH, dt=DT, step=1)
    out = op.integrate(u_0=u, dt=DT, step=3)
    torch.cuda.synchronize()
    print("ncu case done", bool(torch.isfinite(out).all().item()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="fused", choices=["fused", "reference"])
    ap.add_argument("--cpu-samples", type=int, default=16)
    ap.add_argument("--cpu-time-steps", type=int, default=5)
    ap.add_argument("--ncu-case", action="store_true",
                    help="small profiling case: one warm-up step, then 3 time steps of the full batch")
    args = ap.parse_args()
    if args.ncu_case:
        ncu_case()
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
                "cpu_baseline": {k: r[k] for k in ("value", "unit", "cores", "kind", "sample")},
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
    dof_steps = res["B"] * N * N * TIME_STEPS
    value = world * dof_steps / (res["ms"] * 1e-3)
    e2e_value = world * dof_steps / (res["e2e_ms"] * 1e-3)
    peak, peak_kind = _peaks()
    col = res["prof"]["column_pass"]
    achieved = column_pass_bytes(res["B"]) / (col["avg_ms"] * 1e-3) / 1e9 if col["avg_ms"] else None
    cpu = cpu_reference_throughput(min(BATCH, max(os.cpu_count() or 1, args.cpu_samples)), args.cpu_time_steps,
                                   os.cpu_count() or 1)
    line = {
        "metric": METRIC, "value": value, "unit": "DOF*steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/c64", "data": "synthetic (seeded GRF vorticity)",
        "config": {"workload": WORKLOAD, "grid": [N, N], "batch_per_gpu": res["B"], "time_steps": TIME_STEPS,
                   "dt": DT, "nu": 1.0 / RE, "integrator": "SETDRK4 (M=16, r=1)",
                   "parallelism": f"replicas x{world}", "l2": "flushed (256 MB write) between timed steps",
                   "result_finite": res["finite"]},
        "e2e": {"value": e2e_value, "unit": "DOF*steps/s", "h2d_bytes_per_step": res["h2d"],
                "d2h_bytes_per_step": res["d2h"], "ms_per_step": res["e2e_ms"]},
        "gpu_launches": res["launches"] * args.steps,
        "roofline": {"bound": "hbm", "kernel": "k_plane_col (column pass)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": None,
                     "peak_source": f"{peak_kind} hbm_gbs",
                     "per_kernel_ms": {k: v["avg_ms"] for k, v in res["prof"].items() if v["launches"]},
                     "step_model_bytes_per_dof_step": 212,
                     "step_achieved_gbs": 212.0 * dof_steps / world / (res["ms"] * 1e-3) / 1e9 * world},
        "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "clocks": res["clocks"],
    }
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
