"""Hand-written adjoint against the reference's autograd gradients (FP64 golden vectors)."""

import os

import numpy as np
import pytest
import torch

import cases as C
from torchfsm_gb300 import pde
from torchfsm_gb300.operator import Convection, Laplacian

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(C.GRAD_CASES))
@pytest.mark.parametrize("checkpoint", [7, 50])
def test_adjoint_matches_reference_autograd(name, checkpoint):
    from torchfsm_gb300 import adjoint

    c = C.GRAD_CASES[name]
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    dev = torch.device("cuda", 0)
    u0 = torch.tensor(g["u0"], dtype=torch.float32, device=dev, requires_grad=True)
    target = torch.tensor(g["target"], dtype=torch.float32, device=dev)
    nu = torch.tensor(c["nu"], dtype=torch.float32, device=dev, requires_grad=True)
    op = nu * Laplacian() - Convection()
    with torch.no_grad():
        op.integrate(u_0=u0.detach(), mesh=c["mesh"], dt=c["dt"], step=1)
    out = adjoint.integrate_with_grad(op, u0, c["dt"], c["step"], checkpoint=checkpoint)
    loss = ((out - target) ** 2).mean()
    loss.backward()
    assert abs(loss.item() - float(g["loss"])) <= 1e-4 * float(g["loss"])
    gu = u0.grad.double().cpu().numpy()
    err_u = np.linalg.norm(gu - g["grad_u0"]) / np.linalg.norm(g["grad_u0"])
    err_nu = abs(nu.grad.item() - float(g["grad_nu"])) / abs(float(g["grad_nu"]))
    print(f"{name} checkpoint {checkpoint}: grad_u0 rel {err_u:.2e}, grad_nu rel {err_nu:.2e}")
    assert err_u <= 1e-4 and err_nu <= 1e-4


def test_integrate_autograd_entry():
    """op.integrate itself routes to the adjoint when the input or nu requires grad."""
    c = C.GRAD_CASES["grad_burgers1d_n64"]
    g = np.load(os.path.join(GOLDEN, "grad_burgers1d_n64.npz"))
    dev = torch.device("cuda", 0)
    u0 = torch.tensor(g["u0"], dtype=torch.float32, device=dev, requires_grad=True)
    nu = torch.tensor(c["nu"], dtype=torch.float32, device=dev, requires_grad=True)
    op = nu * Laplacian() - Convection()
    out = op.integrate(u_0=u0, mesh=c["mesh"], dt=c["dt"], step=c["step"])
    loss = ((out - torch.tensor(g["target"], dtype=torch.float32, device=dev)) ** 2).mean()
    loss.backward()
    err_nu = abs(nu.grad.item() - float(g["grad_nu"])) / abs(float(g["grad_nu"]))
    assert err_nu <= 1e-4
