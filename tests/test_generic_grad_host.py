"""Gradients of programs outside the hand-written Convection adjoint (vorticity NS, the high-dimensional
KS with its batch-wide mean, KdV with its complex symbol): d loss / d u0 and d loss / d coef against the
reference's float64 autograd (golden vectors), on the CPU. The forward steps through the callback path
with the CPU stand-ins of ``tests/cpu_library.py``; the backward recomputes the segments in torch
arithmetic and differentiates them with autograd (``adjoint._RecomputeFn``)."""

import os

import numpy as np
import pytest
import torch

import cases as C
import cpu_library as CL

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", sorted(C.GENERIC_GRAD_CASES))
def test_gradients_match_reference_autograd(monkeypatch, name):
    case = C.GENERIC_GRAD_CASES[name]
    if case.get("integrator") in C.RK_NAMES:
        pytest.skip("Runge-Kutta steps run through the fused kernels only (test_gpu_adjoint.py)")
    CL.force_callback(monkeypatch)
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    M = C.namespace("torchfsm_gb300")
    coef = torch.tensor(case["coef"], dtype=torch.float32, requires_grad=True)
    op = C.build_generic_grad_op(name, M, coef)
    u0 = torch.tensor(g["u0"], dtype=torch.float32, requires_grad=True)
    target = torch.tensor(g["target"], dtype=torch.float32)
    out = op.integrate(u_0=u0, mesh=case["mesh"], dt=case["dt"], step=case["step"])
    loss = ((out - target) ** 2).mean()
    loss.backward()
    assert abs(loss.item() - float(g["loss"])) <= 1e-4 * abs(float(g["loss"]))
    ref_u = g["grad_u0"]
    err_u = float(np.linalg.norm(u0.grad.numpy() - ref_u) / np.linalg.norm(ref_u))
    err_c = abs(coef.grad.item() - float(g["grad_coef"])) / abs(float(g["grad_coef"]))
    # 1e-4, or twice the reference's own float32 autograd error where that floor is higher (KdV: the
    # i k^3 symbol amplifies every step's rounding; the reference's FP32 gradient is 1.9e-4 off)
    tol_u = max(1e-4, 2 * float(g["fp32_grad_u0_rel_l2"]))
    tol_c = max(1e-4, 2 * float(np.nan_to_num(g["fp32_grad_coef_rel"])))  # NaN: the float32 autograd is NaN
    print(f"{name}: grad u0 rel-L2 {err_u:.2e} (bound {tol_u:.1e}), grad coef rel {err_c:.2e} (bound {tol_c:.1e})")
    assert err_u <= tol_u and err_c <= tol_c


def test_two_segments_equal_one(monkeypatch):
    """Checkpoints every 7 steps (three segments) give the gradients of one 20-step segment."""
    from torchfsm_gb300 import adjoint

    CL.force_callback(monkeypatch)
    case = C.GENERIC_GRAD_CASES["grad_ns2d_n32"]
    M = C.namespace("torchfsm_gb300")
    res = []
    for K in (50, 7):
        coef = torch.tensor(case["coef"], dtype=torch.float32, requires_grad=True)
        op = C.build_generic_grad_op("grad_ns2d_n32", M, coef)
        u0 = torch.tensor(C.generic_grad_initial_condition("grad_ns2d_n32"), dtype=torch.float32, requires_grad=True)
        op.integrate(u_0=u0.detach(), mesh=case["mesh"], dt=case["dt"], step=1)
        with torch.enable_grad():
            out = adjoint._prepare_and_apply(op, u0, case["dt"], case["step"], K)
        (out ** 2).mean().backward()
        res.append((u0.grad.clone(), coef.grad.item()))
    assert torch.allclose(res[0][0], res[1][0], rtol=1e-5, atol=1e-9)
    assert abs(res[0][1] - res[1][1]) <= 1e-5 * abs(res[0][1])


SCHEMES = ["etdrk0", "etdrk1", "etdrk2", "setdrk1", "setdrk2", "setdrk3", "setdrk4"] + list(C.RK_NAMES)


@pytest.mark.parametrize("scheme", SCHEMES)
def test_recomputed_step_of_every_scheme_equals_the_oracle(scheme):
    """The tables and the step the backward pass recomputes (torch, differentiable in L) against the
    oracle's FP64 restatement of the reference's tables and stage recurrences: 1D Burgers spectra on
    64 points, nu = 0.05, dt = 0.01 (RK: 0.005)."""
    import math

    from oracle import spectral as S
    from torchfsm_gb300 import adjoint
    from torchfsm_gb300 import integrator as I

    mesh_info = [(0.0, 2 * math.pi, 64)]
    om = S.OMesh(mesh_info)
    lin = S.linear_symbol(om, [(0.05, ("laplacian",))], 1)
    nl = S.make_nonlinear(om, [(-1.0, "convection")])
    dt = 0.005 if scheme in C.RK_NAMES else 0.01
    u = om.fft(C._bl(11, (64,), 4, 0.5)(mesh_info, 2, 1))
    linear_only = scheme == "etdrk0"
    ref = S.stage_step(scheme, S.build_tables(scheme, lin, dt), None if linear_only else nl, u)
    if scheme in C.RK_NAMES:
        code = int(I.RKIntegrator[scheme].value)
    elif scheme.startswith("setdrk"):
        code = int(I.SETDRKIntegrator[scheme.upper()].value)
    else:
        code = int(I.ETDRKIntegrator[scheme.upper()].value)
    L = torch.tensor(lin, dtype=torch.complex128)
    tabs = adjoint._scheme_tables(code, L, dt, 16, 1.0)

    def nonlinear(x):
        return torch.tensor(nl(x.numpy()))

    out = adjoint._scheme_step(code, torch.tensor(u), tabs, None if linear_only else nonlinear, dt).numpy()
    err = float(np.linalg.norm(out - ref) / np.linalg.norm(ref))
    assert err < 1e-12, (scheme, err)


def test_table_derivatives_are_those_of_the_contour_formulas():
    """The analytic d(table)/dL of the hand-written adjoint against torch autograd through the same
    FP64 contour means, over symbols from 0 to -1e4 at dt = 1e-3 and 0.05 (central differences in
    FP64 agree only to 1e-5 here: at dt = 1e-3 the c6 table is 1e-12 and its differences cancel)."""
    from torchfsm_gb300 import adjoint

    Lr = -torch.cat([torch.zeros(1), torch.logspace(-3, 4, 60)]).to(torch.float64)
    for dt in (1e-3, 0.05):
        ana = adjoint._table_derivatives(Lr.to(torch.complex128), dt, 16, 1.0)
        x = Lr.clone().requires_grad_(True)
        tabs = adjoint._contour_tables(x.to(torch.complex128), dt, 16, 1.0)
        for t, (a, tab) in enumerate(zip(ana, tabs)):
            (g,) = torch.autograd.grad(tab.sum(), x, retain_graph=True)
            err = float((a - g).abs().max() / g.abs().max())
            assert err < 1e-10, (dt, t, err)
