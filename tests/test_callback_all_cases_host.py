"""The callback path on every fused golden case (CPU).

The callback path (``integrator/_callback.py``) steps programs whose nonlinear terms have no
fused kernel. Here it is forced onto the programs that do have one -- Burgers 1D/2D/3D, 2D
vorticity NS, KS with the batch-wide mean, KdV with its complex Nyquist mode, 3D velocity NS
with the Leray projection, explicit sources, batched coefficients, ETDRK1/2 and SETDRK1-4 -- by
making the lowering refuse every nonlinear term, and run through ``integrate`` on the CPU
stand-ins of ``tests/cpu_library.py``. Its results must meet the same bar as the fused kernels
against the reference's float64 runs: relative L2 <= 1e-5 over the recorded trajectory. Cases of
the Runge-Kutta schemes (not offered on the callback path) are left out.
"""

import os

import numpy as np
import pytest
import torch

import cases as C
import cpu_library as CL
from oracle import spectral as S
from torchfsm_gb300.integrator._callback import CallbackPlan

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-5
NAMES = sorted(n for n, c in C.CASES.items() if c.get("integrator") not in C.RK_NAMES)


@pytest.fixture
def callback_everywhere(monkeypatch):
    CL.force_callback(monkeypatch)


@pytest.mark.parametrize("name", NAMES)
def test_callback_path_matches_reference_fp64(name, callback_everywhere):
    case = C.CASES[name]
    M = C.namespace("torchfsm_gb300")
    op = case["build"](M)
    if case.get("integrator"):
        C.set_case_integrator(op, M, case["integrator"])
    u0 = torch.tensor(C.initial_condition(name), dtype=torch.float32)
    rec_fn = C.record_fn(name)
    rec = M.traj_recorder.AutoRecorder(control_func=rec_fn) if rec_fn is not None else None
    out = op.integrate(u_0=u0, mesh=case["mesh"], dt=case["dt"], step=case["step"], trajectory_recorder=rec)
    if case["nl"]:
        assert isinstance(op._state_dict["integrator"].plan, CallbackPlan)
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    ref = g["traj"] if rec is not None else g["final"]
    assert tuple(out.shape) == ref.shape
    assert S.rel_l2(out.numpy(), ref) <= TOL
