"""Host-side figures of bench.py (no GPU)."""

import math

import bench


def test_fft_flop_fraction_of_the_1d_solve():
    r = bench.fft_flop_fraction(128, 1, 200, 1.0)
    # 12 real transforms of 2.5 n log2 n flops per step: 30 log2 n flops per DOF*step
    assert r["fft_flops_per_dof_step"] == 30 * 7
    assert math.isclose(r["achieved_tflops"], 210 * 128 * 200 / 1e-3 / 1e12)
    assert math.isclose(r["peak_tflops"], 152 * 128 * 2 * 2.07e3 / 1e6)
    assert math.isclose(r["frac"], r["achieved_tflops"] / r["peak_tflops"])


def test_fp64_accuracy_leg_runs_the_reference_in_float64():
    """The accuracy leg of the headline line integrates with the reference itself in float64: on the
    CPU, at 32^2, its result equals the oracle's FP64 integration of the same vorticity to 1e-10, and an
    FP32 run of the same reference lands inside the 1e-5 parity bar but not at FP64 round-off."""
    import numpy as np
    import pytest
    import torch

    R, why = bench._import_reference()
    if R is None:
        pytest.skip(why)
    from oracle import spectral as S
    from torchfsm_gb300 import initial

    mesh = [(0.0, 2 * math.pi, 32)] * 2
    w0 = initial.gaussian_random_field((32, 32), 2, 1, initial.vorticity_spectrum, 5)
    w0 = w0 if w0.ndim == 4 else w0[:, None]
    steps, dt = 20, 1e-3
    ref64, _ = S.integrate(w0, mesh, [(1e-3, ("laplacian",))], [(-1.0, "vorticity_convection")], dt, steps)

    def make(R):
        return R.pde.NavierStokesVorticity(1000.0)

    r = bench.fp64_reference_rel_l2(make, mesh, w0, dt, steps, ref64, "cpu")
    assert r["samples"] == 2 and r["steps"] == steps
    assert r["rel_l2"] < 1e-10, r
    ours32 = make(R).integrate(u_0=torch.tensor(w0, dtype=torch.float32), mesh=mesh, dt=dt, step=steps)
    r32 = bench.fp64_reference_rel_l2(make, mesh, w0, dt, steps, ours32, "cpu")
    assert 1e-9 < r32["rel_l2"] < 1e-5, r32


def test_accuracy_by_step_compares_ours_and_the_reference_fp32_with_fp64():
    """The per-step accuracy leg: the oracle's FP64 results stand in for ours and land at FP64
    round-off of the reference's float64 run at every checkpoint; the reference's own float32 run
    lands inside the 1e-5 bar but above round-off; the energy-spectrum figure is reported."""
    import numpy as np
    import pytest

    R, why = bench._import_reference()
    if R is None:
        pytest.skip(why)
    from oracle import spectral as S
    from torchfsm_gb300 import initial

    mesh = [(0.0, 2 * math.pi, 32)] * 2
    w0 = initial.gaussian_random_field((32, 32), 2, 1, initial.vorticity_spectrum, 5)
    w0 = w0 if w0.ndim == 4 else w0[:, None]
    dt = 1e-3
    ours = {}
    for k in (4, 12):
        ours[k], _ = S.integrate(w0, mesh, [(1e-3, ("laplacian",))], [(-1.0, "vorticity_convection")], dt, k)
    r = bench.accuracy_by_step(lambda R: R.pde.NavierStokesVorticity(1000.0), mesh, w0, dt, (4, 12), ours, "cpu")
    assert set(r["by_step"]) == {"4", "12"} and set(r["reference_fp32_by_step"]) == {"4", "12"}, r
    assert max(r["by_step"].values()) < 1e-10, r
    assert r["rel_l2"] == r["by_step"]["12"]
    assert all(1e-9 < v < 1e-5 for v in r["reference_fp32_by_step"].values()), r
    assert r["energy_spectrum_max_rel_diff"] < 1e-8, r


def test_fp64_accuracy_leg_reports_failure_instead_of_raising():
    import numpy as np
    import pytest

    R, why = bench._import_reference()
    if R is None:
        pytest.skip(why)

    def broken(R):
        raise RuntimeError("no such operator")

    r = bench.fp64_reference_rel_l2(broken, [(0.0, 1.0, 8)], np.zeros((1, 1, 8)), 0.1, 1, np.zeros((1, 1, 8)), "cpu")
    assert "unavailable" in r and "no such operator" in r["unavailable"]


def test_reference_request_sample_runs_the_reference_on_the_cheapest_requests():
    import numpy as np
    import pytest
    import torch

    R, why = bench._import_reference()
    if R is None:
        pytest.skip(why)
    from torchfsm_gb300.serving import SolveRequest

    rng = np.random.default_rng(3)
    reqs = [
        SolveRequest(0, "ks1d", 256, 1, 6, 0.05, torch.tensor(rng.standard_normal((1, 1, 256)), dtype=torch.float32)),
        SolveRequest(1, "burgers2d", 64, 1, 3, 0.02,
                     torch.tensor(0.25 * rng.standard_normal((1, 2, 64, 64)), dtype=torch.float32)),
        SolveRequest(2, "ks1d", 512, 2, 50, 0.05, torch.zeros(2, 1, 512)),
    ]
    r = bench.reference_request_sample(reqs, "cpu", 2)
    assert r["requests"] == 2 and sorted(r["rids"]) == [0, 1]  # the two cheapest
    assert r["value"] > 0 and r["unit"] == "DOF*steps/s"
    assert r["max_rel_l2_served_vs_reference_fp32"] == {}  # no served results yet


def test_energy_spectrum_of_single_modes():
    import torch

    n = 32
    x = torch.arange(n, dtype=torch.float64) / n * 2 * math.pi
    u = (torch.cos(3 * x) + 2 * torch.sin(5 * x)).reshape(1, 1, n)
    e = bench.energy_spectrum(u)
    # |u_hat(+-k)| = n a / 2 for amplitude a: shell k holds a^2 / 2
    assert math.isclose(float(e[3]), 0.5, rel_tol=1e-12) and math.isclose(float(e[5]), 2.0, rel_tol=1e-12)
    assert float(e.sum()) == float(e[3] + e[5])
    # Parseval: the shells sum to the mean square of the field
    assert math.isclose(float(e.sum()), float((u ** 2).mean()), rel_tol=1e-12)
    v = torch.cos(x.reshape(n, 1) + 2 * x.reshape(1, n)).reshape(1, 1, n, n).repeat(2, 2, 1, 1)
    e2 = bench.energy_spectrum(v)  # |k| = sqrt(5) -> shell 2, two channels
    assert math.isclose(float(e2[2]), 1.0, rel_tol=1e-12) and math.isclose(float(e2.sum()), 1.0, rel_tol=1e-12)


def test_reference_cpu_leg_times_the_reference_package():
    import pytest

    R, why = bench._import_reference()
    if R is None:
        pytest.skip(why)
    r = bench.reference_cpu_throughput(1, k1=1, k2=2, threads=2)
    assert r["value"] > 0 and r["cores"] == 2 and r["unit"] == "DOF*steps/s"
    assert "torch CPU" in r["kind"]


def test_reference_arm_prints_one_line_with_the_contract_keys():
    import json
    import os
    import subprocess
    import sys

    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    cmd = [sys.executable, os.path.join(repo, "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
           "--cpu-samples", "1", "--cpu-time-steps", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=600, cwd=repo)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["unit"] == "DOF*steps/s" and line["higher_is_better"] is True
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    # under torchrun only rank 0 runs and prints
    env.update(RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=600, cwd=repo)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_fused_line_from_measurements():
    import json
    from types import SimpleNamespace

    prof = {"column_pass": {"avg_ms": 0.06, "launches": 4000}, "row_pass": {"avg_ms": 0.024, "launches": 4000},
            "prime": {"avg_ms": 0.05, "launches": 1}, "other": {"avg_ms": 0.0, "launches": 0}}
    res = {"ms": 250.0, "e2e_ms": 251.0, "finite": True, "clocks": {"sm_mhz": 2070.0}, "launches": 64008,
           "prof": prof, "h2d": 16777216, "d2h": 16777216, "B": 64,
           "torch_ref": {"value": 1.7e9}, "fp64": {"rel_l2": 3e-7}, "first_ms": 400.0}
    args = SimpleNamespace(steps=5, warmup=3)
    cpu = {"value": 1.8e7, "unit": "DOF*steps/s", "cores": 16, "kind": "port", "sample": "s", "seconds": 1.0}
    ref_cpu = {"value": 2.0e7}
    line = bench.fused_line(res, args, 1, cpu, ref_cpu)
    json.dumps(line)
    dof_steps = 64 * 256 * 256 * 1000
    assert math.isclose(line["value"], dof_steps / 0.25)
    assert math.isclose(line["e2e"]["value"], dof_steps / 0.251)
    assert line["e2e"]["first_call_with_build_ms"] == 400.0
    assert line["config"]["rel_l2_vs_fp64"] == 3e-7 and line["accuracy_vs_fp64"] == {"rel_l2": 3e-7}
    assert line["gpu_launches"] == 64008 * 5
    assert math.isclose(line["roofline"]["achieved"], bench.column_pass_bytes(64) / 0.06e-3 / 1e9)
    assert math.isclose(line["roofline"]["frac"], line["roofline"]["achieved"] / line["roofline"]["peak"])
    assert set(line["roofline"]["per_kernel_ms"]) == {"column_pass", "row_pass", "prime"}
    assert line["cpu_baseline"] == {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    assert math.isclose(line["torch_gpu_reference"]["fused_e2e_over_reference"], line["e2e"]["value"] / 1.7e9)
    assert math.isclose(line["reference_cpu"]["fused_e2e_over_reference_cpu"], line["e2e"]["value"] / 2.0e7)
    # N > 1: no CPU baselines, value is the whole job's
    res2 = dict(res, torch_ref=None, fp64=None)
    line2 = bench.fused_line(res2, args, 2, None, None)
    assert line2["cpu_baseline"] is None and line2["reference_cpu"] is None
    assert math.isclose(line2["value"], 2 * dof_steps / 0.25) and line2["config"]["rel_l2_vs_fp64"] is None


def test_other_workloads_summaries_and_failures(monkeypatch):
    """The headline line's summaries of the other workloads: the named keys of each leg's own line,
    run with few repetitions, and a failing leg reported instead of raised."""
    import argparse

    seen = {}

    def fake_1d(args):
        seen["steps"], seen["warmup"] = args.steps, args.warmup
        return {"value": 1.0, "unit": "DOF*steps/s", "latency_ms": {"p50": 2.0}, "config": {"rel_l2_traj_vs_fp64": 3e-7}}

    def broken(args):
        raise RuntimeError("no GPU")

    def fake_serving(args):
        seen["serve"] = (args.requests, args.loads, args.ref_requests, args.ref_cpu_requests)
        return {"value": 5.0, "unit": "DOF*steps/s", "serving": {"speedup_vs_plain": 3.2, "latency_s": {"p99": 0.8}}}

    monkeypatch.setattr(bench, "run_burgers1d", fake_1d)
    monkeypatch.setattr(bench, "run_burgers3d", broken)
    monkeypatch.setattr(bench, "run_burgers2d_grad", broken)
    monkeypatch.setattr(bench, "run_serving", fake_serving)
    out = bench.other_workloads(argparse.Namespace(steps=20, warmup=5, no_fp64_reference=False,
                                                   serve_summary_requests=300, load=0.25, loads="0.25,0.35"))
    serve = out["serving_300_requests"]
    assert serve["value"] == 5.0 and serve["serving.speedup_vs_plain"] == 3.2 and serve["serving.latency_s"] == {"p99": 0.8}
    assert seen["serve"] == (300, "0.25,0.35", 0, 0)  # the Poisson loads, no reference samples
    one = out["burgers1d_n128_200steps"]
    assert one["value"] == 1.0 and one["latency_ms"] == {"p50": 2.0} and one["config.rel_l2_traj_vs_fp64"] == 3e-7
    assert one["torch_gpu_reference.latency_ms"] is None and one["wall_s"] >= 0
    assert (seen["steps"], seen["warmup"]) == (3, 1)
    assert "no GPU" in out["burgers3d_256cubed_200steps"]["unavailable"]
    assert "no GPU" in out["burgers2d_grad_128x128_b16_500steps"]["unavailable"]
