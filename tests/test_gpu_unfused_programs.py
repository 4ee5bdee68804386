"""GPU parity of programs without a fused kernel (stepped through their Python callables).

``Operator.integrate`` of a program with a Python-callable ``ImplicitSource(f)``, the conservative
convection form, or two kinds of nonlinear term with an explicit source, on a CUDA device: the
library's coefficient tables and transforms with the cores called on the device, against the
reference's float64 runs (golden vectors). Tolerance: relative L2 <= 1e-5 over the whole recorded
trajectory where one is recorded. ``tests/test_callback_host.py`` runs the same cases on the CPU
with stand-ins for the two library pieces.
"""

import os

import numpy as np
import pytest
import torch

import cases as C
from oracle import spectral as S
from torchfsm_gb300.integrator._callback import CallbackPlan

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-5
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(C.CALLBACK_CASES))
def test_callback_program_matches_reference_fp64(name):
    case = C.CALLBACK_CASES[name]
    M = C.namespace("torchfsm_gb300")
    op = case["build"](M)
    if case.get("integrator"):
        C.set_case_integrator(op, M, case["integrator"])
    u0 = torch.tensor(C.initial_condition(name), dtype=torch.float32, device="cuda")
    rec_fn = C.record_fn(name)
    rec = M.traj_recorder.AutoRecorder(control_func=rec_fn) if rec_fn is not None else None
    out = op.integrate(u_0=u0, mesh=case["mesh"], dt=case["dt"], step=case["step"], trajectory_recorder=rec)
    assert isinstance(op._state_dict["integrator"].plan, CallbackPlan)
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    ref = g["traj"] if rec is not None else g["final"]
    got = out.cpu().numpy()
    assert got.shape == ref.shape
    assert S.rel_l2(got, ref) <= TOL
