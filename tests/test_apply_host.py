"""One-shot evaluation with the torch cores, in float64 on the CPU, against the reference.

Every ``APPLY_CASES`` program (the pde constructors, Grad/Div/Curl, the velocity and pressure
post-processing operators, ``functional.*``, ``LinearOperator.solve``) is evaluated through the
public API with its cores' torch arithmetic -- the arithmetic of the callback path and of the
channel-changing post-processing operators -- by switching off the fused FSM_APPLY evaluation
(which needs a GPU; ``tests/test_gpu_apply.py`` covers it). In float64 the results must equal the
reference's float64 results (golden vectors) to 1e-10: this pins the operator algebra
(coefficients, signs, term kinds) and every core's formula.
"""

import os

import numpy as np
import pytest
import torch

import cases as C
from oracle import spectral as S
from torchfsm_gb300.operator import _base as B

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", sorted(C.APPLY_CASES))
def test_torch_cores_match_reference_fp64(name, monkeypatch):
    monkeypatch.setattr(B.OperatorLike, "_apply_fused", lambda self, u, u_fft: None)
    case = C.APPLY_CASES[name]
    M = C.namespace("torchfsm_gb300")
    u = torch.tensor(C.apply_input(name), dtype=torch.float64)
    out = case["fn"](M, u, case["mesh"])
    ref = np.load(os.path.join(GOLDEN, f"{name}.npz"))["out"]
    assert tuple(out.shape) == ref.shape
    assert S.rel_l2(out.numpy(), ref) <= 1e-10
