"""Programs without a fused kernel, stepped through their Python callables, on the CPU.

``Operator.integrate`` of a program whose nonlinear terms have no CUDA kernel (a Python-callable
``ImplicitSource(f)``, ``ConservativeConvection``, two kinds of nonlinear term with an explicit
source) builds a library plan of the linear part and a ``CallbackPlan`` around it. These tests run
that whole path through the public API with the two device pieces replaced by CPU stand-ins:

* the plan's coefficient tables are the oracle's FP64 tables of the same linear symbol, laid out
  as the library lays them out (``fsm_plan_tables``: [tables][lin_batch][lin_channel][half
  spectrum], per scheme E, E2, c1.. in the library's order);
* the forward and inverse transforms are torch's real FFTs.

The results are compared with the reference's float64 runs of the same programs (golden
vectors made by ``tests/golden/make_golden.py``), at the GPU parity bar: relative L2 <= 1e-5 over
the whole recorded trajectory.
"""

import os

import numpy as np
import pytest
import torch

import cases as C
from oracle import spectral as S
from torchfsm_gb300 import _lib, _native
from torchfsm_gb300.integrator._callback import CallbackPlan

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-5
_RealSpectral = _native.Spectral


def _library_tables(integrator: int, lin: np.ndarray, dt: float, m: int, r: float) -> list:
    """The scheme's tables in the library's order (oracle values, FP64)."""
    if integrator in (_lib.FSM_ETDRK1, _lib.FSM_ETDRK2):
        t = S.etdrk_coefs(1 if integrator == _lib.FSM_ETDRK1 else 2, lin, dt)
        keys = ["E", "c1"] + (["c2"] if integrator == _lib.FSM_ETDRK2 else [])
    else:
        order = {_lib.FSM_SETDRK1: 1, _lib.FSM_SETDRK2: 2, _lib.FSM_SETDRK3: 3, _lib.FSM_SETDRK4: 4}[integrator]
        t = S.setdrk_coefs(order, lin, dt, m, r)
        keys = {1: ["E", "c1"], 2: ["E", "c1", "c2"], 3: ["E", "E2", "c1", "c2", "c3", "c4", "c5"],
                4: ["E", "E2", "c1", "c4", "c5", "c6"]}[order]
    return [np.broadcast_to(np.asarray(t[k], dtype=np.complex128), lin.shape) for k in keys]


class _CpuLinearPlan:
    """Stands in for the library plan of a linear part (same constructor as NativePlan)."""

    def __init__(self, program, dt, integrator, device, n_integration_points=16, integration_radius=1.0,
                 linear_coef64=None, table_batch=0):
        assert program.nonlinear == _lib.FSM_NL_NONE and not program.sources
        self.program, self.dt, self.integrator = program, float(dt), integrator
        self.device = torch.device(device)
        self.shape = program.shape
        self.n_channel = program.n_channel
        self.handle = None
        nd = len(self.shape)
        h = self.shape[-1] // 2 + 1
        if linear_coef64 is None:
            lin = np.zeros((1, 1) + self.shape[:-1] + (h,), dtype=np.complex128)
        else:
            L = linear_coef64
            if L.dim() != nd + 2:
                L = L.reshape((1, 1) + tuple(L.shape[-nd:]))
            L = L.expand(tuple(L.shape[:2]) + self.shape)
            lin = L[..., :h].cpu().numpy().astype(np.complex128)
        self.lin_batch = lin.shape[0]
        self._tables = np.stack([t.reshape(-1) for t in _library_tables(
            integrator, lin, self.dt, n_integration_points, integration_radius)])

    def tables(self):
        return torch.from_numpy(self._tables.astype(np.complex64))


class _CpuSpectral(_RealSpectral):
    """torch's real FFTs in place of the library's transforms."""

    def to_half(self, u):
        nd = len(self.shape)
        return torch.fft.rfftn(u.to(torch.float32), dim=tuple(range(-nd, 0))).to(torch.complex64)

    def to_physical(self, half, keep_input=True):
        nd = len(self.shape)
        return torch.fft.irfftn(half, s=self.shape, dim=tuple(range(-nd, 0))).to(torch.float32)


@pytest.fixture
def cpu_library(monkeypatch):
    monkeypatch.setattr(_native, "NativePlan", _CpuLinearPlan)
    monkeypatch.setattr(_native, "Spectral", _CpuSpectral)
    monkeypatch.setattr(_native, "_require_cuda", lambda t, what: None)


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


def test_gradients_of_a_callback_program_are_not_provided(cpu_library):
    M = C.namespace("torchfsm_gb300")
    op = 0.05 * M.operator.Laplacian() + M.operator.ImplicitSource(lambda u: u - u ** 3)
    u0 = torch.rand(1, 1, 64, requires_grad=True)
    with pytest.raises(NotImplementedError, match="Python callables"):
        op.integrate(u_0=u0, mesh=[(0, 1, 64)], dt=0.01, step=2)


def test_linear_part_that_changes_channels_stays_unsupported(cpu_library):
    M = C.namespace("torchfsm_gb300")
    op = M.operator.Grad() + M.operator.ImplicitSource(lambda u: u ** 2)
    with pytest.raises((_lib.UnsupportedProgram, ValueError)):
        op.integrate(u_0=torch.rand(1, 1, 16, 16), mesh=[(0, 1, 16), (0, 1, 16)], dt=0.01, step=1)
