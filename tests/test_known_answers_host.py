"""Known answers of the spectral operators, derived from calculus (CPU, float64).

The reference validates its operators in a documentation notebook by applying them to sines
and cosines on the 3D mesh [(0, 2 pi, 32), (0, 4 pi, 64), (0, 8 pi, 128)] and comparing with
the closed-form derivatives. The same checks here, written from the mathematics: the symbols
the library's coefficient tables are built from (Laplacian, Biharmonic, SpatialDerivative), and
the torch cores of the one-shot and callback paths (Grad, Div, Curl, Convection,
ConservativeConvection). Every field holds wavenumbers well inside the 2/3 cut, and every
product stays inside it, so the answers are exact to rounding.
"""

import math

import pytest
import torch

from torchfsm_gb300.mesh import FourierMesh, MeshGrid
from torchfsm_gb300.operator import (Biharmonic, ConservativeConvection, Curl, Div, Grad, Laplacian,
                                     SpatialDerivative)
from torchfsm_gb300.operator.generic._convection import _ConvectionCore

MESH3 = [(0, 2 * math.pi, 32), (0, 4 * math.pi, 64), (0, 8 * math.pi, 128)]
TOL = 1e-10


def _grids(mesh_info):
    g = MeshGrid(mesh_info, dtype=torch.float64).mesh_grid()
    return [t.reshape(1, 1, *t.shape) for t in (g if isinstance(g, (list, tuple)) else [g])]


def _close(a, b):
    scale = max(float(b.abs().max()), 1.0)
    assert float((a - b).abs().max()) <= TOL * scale


def _apply_symbol(op, u, mesh_info):
    """ifft(L * fft(u)).real with the operator's registered symbol L (its linear coefficient)."""
    fm = FourierMesh(mesh_info, dtype=torch.float64)
    op.register_mesh(fm, u.shape[1])
    return fm.ifft(op.linear_coef * fm.fft(u)).real


def _vector(*parts):
    return torch.cat(parts, dim=1)


def test_laplacian_of_sines_and_cosines():
    x, y, z = _grids(MESH3)
    u = _vector(torch.sin(x), torch.cos(y), torch.sin(z) + torch.cos(z))
    _close(_apply_symbol(Laplacian(), u, MESH3), -u)
    f = torch.sin(2 * x) * torch.cos(y)
    _close(_apply_symbol(Laplacian(), f, MESH3), -5 * f)


def test_biharmonic():
    x, y, z = _grids(MESH3)
    f = torch.sin(x) * torch.cos(y)
    _close(_apply_symbol(Biharmonic(), f, MESH3), 4 * f)
    g = torch.cos(3 * z)
    _close(_apply_symbol(Biharmonic(), g, MESH3), 81 * g)


@pytest.mark.parametrize("dim,order", [(0, 1), (0, 2), (1, 3), (2, 1), (2, 4)])
def test_spatial_derivative(dim, order):
    grids = _grids(MESH3)
    k = [2, 1, 3][dim]
    f = torch.sin(k * grids[dim])
    # d^n/dx^n sin(k x) = k^n sin(k x + n pi / 2)
    want = k ** order * torch.sin(k * grids[dim] + order * math.pi / 2)
    _close(_apply_symbol(SpatialDerivative(dim, order), f, MESH3), want)


def test_grad_of_a_product():
    x, y, z = _grids(MESH3)
    f = torch.sin(x) * torch.cos(y) * torch.sin(z)
    got = Grad()(f, mesh=MESH3)
    want = _vector(torch.cos(x) * torch.cos(y) * torch.sin(z), -torch.sin(x) * torch.sin(y) * torch.sin(z),
                   torch.sin(x) * torch.cos(y) * torch.cos(z))
    _close(got, want)


def test_div():
    x, y, z = _grids(MESH3)
    u = _vector(torch.sin(x), torch.cos(y), torch.sin(z) + torch.cos(z))
    got = Div()(u, mesh=MESH3)
    _close(got, torch.cos(x) - torch.sin(y) + torch.cos(z) - torch.sin(z))


def test_curl_3d_and_2d():
    x, y, z = _grids(MESH3)
    u = _vector(torch.sin(y), torch.sin(z), torch.sin(x))
    _close(Curl()(u, mesh=MESH3), _vector(-torch.cos(z), -torch.cos(x), -torch.cos(y)))
    mesh2 = MESH3[:2]
    x2, y2 = _grids(mesh2)
    v = _vector(torch.sin(y2), torch.sin(x2))
    _close(Curl()(v, mesh=mesh2), torch.cos(x2) - torch.cos(y2))


def test_convection_and_its_conservative_form():
    x, y, z = _grids(MESH3)
    w = torch.sin(z) + torch.cos(z)
    dw = torch.cos(z) - torch.sin(z)
    u = _vector(torch.sin(x), torch.cos(y), w)
    fm = FourierMesh(MESH3, dtype=torch.float64)
    # (u . grad) u: each component depends on its own axis only
    adv = fm.ifft(_ConvectionCore()(fm.fft(u), fm, u)).real
    _close(adv, _vector(torch.sin(x) * torch.cos(x), -torch.cos(y) * torch.sin(y), w * dw))
    # div(u u) = (u . grad) u + u div(u)
    div = torch.cos(x) - torch.sin(y) + dw
    cons = ConservativeConvection()(u, mesh=MESH3)
    _close(cons, adv + u * div)


def test_two_thirds_rule_on_ten_points():
    # N = 10: |k| <= 5, the 2/3 cut keeps |k| <= 10/3, so sin 4x is removed and sin 2x kept
    fm = FourierMesh([(0, 2 * math.pi, 10)], dtype=torch.float64)
    (x,) = _grids([(0, 2 * math.pi, 10)])
    u = torch.sin(2 * x) + torch.sin(4 * x)
    kept = fm.ifft(fm.fft(u) * fm.low_pass_filter(2 / 3)).real
    _close(kept, torch.sin(2 * x))
