"""Programs without a fused kernel, stepped through their Python callables, on the CPU.

``Operator.integrate`` of a program whose nonlinear terms have no CUDA kernel (a Python-callable
``ImplicitSource(f)``, ``ConservativeConvection``, two kinds of nonlinear term with an explicit
source) builds a library plan of the linear part and a ``CallbackPlan`` around it. These tests run
that whole path through the public API with the two device pieces (the plan's coefficient
tables and the transforms) replaced by the CPU stand-ins of ``tests/cpu_library.py``.

The results are compared with the reference's float64 runs of the same programs (golden
vectors made by ``tests/golden/make_golden.py``), at the GPU parity bar: relative L2 <= 1e-5 over
the whole recorded trajectory.
"""

import os

import numpy as np
import pytest
import torch

import cases as C
import cpu_library as CL
from oracle import spectral as S
from torchfsm_gb300 import _lib
from torchfsm_gb300.integrator._callback import CallbackPlan

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-5


@pytest.fixture
def cpu_library(monkeypatch):
    CL.install(monkeypatch)


def _run(name):
    case = C.CALLBACK_CASES[name]
    M = C.namespace("torchfsm_gb300")
    op = case["build"](M)
    if case.get("integrator"):
        C.set_case_integrator(op, M, case["integrator"])
    u0 = torch.tensor(C.initial_condition(name), dtype=torch.float32)
    rec_fn = C.record_fn(name)
    rec = M.traj_recorder.AutoRecorder(control_func=rec_fn) if rec_fn is not None else None
    out = op.integrate(u_0=u0, mesh=case["mesh"], dt=case["dt"], step=case["step"], trajectory_recorder=rec)
    return op, out, rec is not None


@pytest.mark.parametrize("name", sorted(C.CALLBACK_CASES))
def test_callback_program_matches_reference_fp64(name, cpu_library):
    op, out, recorded = _run(name)
    assert isinstance(op._state_dict["integrator"].plan, CallbackPlan)
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    ref = g["traj"] if recorded else g["final"]
    assert out.shape == ref.shape
    assert S.rel_l2(out.numpy(), ref) <= TOL


def test_launch_count_and_recorded_frames(cpu_library):
    op, out, recorded = _run("allencahn1d_n64")
    plan = op._state_dict["integrator"].plan
    # one dealiased inverse transform per nonlinear evaluation, four evaluations per SETDRK4 step
    assert plan.launch_count(10) == 40
    assert recorded and out.shape[1] == 100 // 20 + 1


def test_runge_kutta_with_a_python_callable_is_unsupported(cpu_library):
    M = C.namespace("torchfsm_gb300")
    op = M.operator.Laplacian() + M.operator.ImplicitSource(lambda u: u ** 2)
    op.set_integrator(M.integrator.RKIntegrator.RK4)
    with pytest.raises(_lib.UnsupportedProgram, match="Runge-Kutta"):
        op.integrate(u_0=torch.rand(1, 1, 64), mesh=[(0, 1, 64)], dt=0.01, step=2)


def test_gradients_of_a_callback_program_match_central_differences(cpu_library):
    """A program with a Python-callable term: its gradient (segments recomputed in torch arithmetic
    and differentiated by autograd) against central differences of the same integration."""
    M = C.namespace("torchfsm_gb300")
    op = 0.05 * M.operator.Laplacian() + M.operator.ImplicitSource(lambda u: u - u ** 3)
    mesh = [(0, 1, 64)]
    u0 = torch.tensor(C.initial_condition("allencahn1d_n64")[:1], dtype=torch.float32)
    target = torch.zeros_like(u0)

    def loss_of(u):
        return ((op.integrate(u_0=u, mesh=mesh, dt=0.01, step=12) - target) ** 2).mean()

    x = u0.clone().requires_grad_(True)
    loss_of(x).backward()
    v = torch.tensor(np.random.default_rng(3).standard_normal(u0.shape), dtype=torch.float32)
    v /= v.norm()
    eps = 1e-2
    with torch.no_grad():
        fd = (loss_of(u0 + eps * v) - loss_of(u0 - eps * v)).item() / (2 * eps)
    ad = float((x.grad * v).sum())
    assert abs(fd - ad) <= 2e-2 * abs(ad), (fd, ad)


def test_linear_part_that_changes_channels_stays_unsupported(cpu_library):
    M = C.namespace("torchfsm_gb300")
    op = M.operator.Grad() + M.operator.ImplicitSource(lambda u: u ** 2)
    with pytest.raises((_lib.UnsupportedProgram, ValueError)):
        op.integrate(u_0=torch.rand(1, 1, 16, 16), mesh=[(0, 1, 16), (0, 1, 16)], dt=0.01, step=1)


def test_batched_linear_coefficient_matches_samples_run_alone(cpu_library):
    """A tensor coefficient [B, 1, 1] on the linear term gives one table entry per sample."""
    M = C.namespace("torchfsm_gb300")
    u0 = torch.tensor(C.initial_condition("allencahn1d_n64"), dtype=torch.float32)
    mesh = [(0, 2 * np.pi, 64)]
    nus = torch.tensor([0.05, 0.2], dtype=torch.float32).reshape(2, 1, 1)
    op = nus * M.operator.Laplacian() + M.operator.ImplicitSource(C._allen_cahn_source)
    both = op.integrate(u_0=u0, mesh=mesh, dt=0.01, step=40)
    plan = op._state_dict["integrator"].plan
    assert plan.tables.shape[1] == 2  # lin_batch
    for b in range(2):
        alone_op = float(nus[b]) * M.operator.Laplacian() + M.operator.ImplicitSource(C._allen_cahn_source)
        alone = alone_op.integrate(u_0=u0[b : b + 1], mesh=mesh, dt=0.01, step=40)
        assert S.rel_l2(both[b : b + 1].numpy(), alone.numpy()) <= 1e-6


def test_per_sample_coefficient_on_a_nonlinear_term(cpu_library):
    """A tensor coefficient [B, 1, 1] on the convection term (no fused kernel takes it) steps
    through the callback path; each sample equals the FP64 oracle's run with its own scalar."""
    M = C.namespace("torchfsm_gb300")
    u0 = torch.tensor(C.initial_condition("allencahn1d_n64"), dtype=torch.float32)
    mesh = [(0, 2 * np.pi, 64)]
    coefs = torch.tensor([1.0, 0.5]).reshape(2, 1, 1)
    op = 0.05 * M.operator.Laplacian() - coefs * M.operator.Convection()
    both = op.integrate(u_0=u0, mesh=mesh, dt=0.01, step=30)
    assert isinstance(op._state_dict["integrator"].plan, CallbackPlan)
    for b in range(2):
        ref, _ = S.integrate(u0[b : b + 1].double().numpy(), mesh, [(0.05, ("laplacian",))],
                             [(-float(coefs[b]), "convection")], 0.01, 30)
        assert S.rel_l2(both[b : b + 1].numpy(), ref) <= TOL
