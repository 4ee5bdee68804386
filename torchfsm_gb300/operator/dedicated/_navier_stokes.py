"""Navier-Stokes nonlinear terms (operator/dedicated/_navier_stokes.py).

VorticityConvection: u . grad(w) with u = (d_y psi, -d_x psi), psi = -w/lap
(2D scalar vorticity). NSPressureConvection: -grad p - (u . grad) u with the
pressure from the Leray projection p = lap^-1 div((u . grad) u) (optionally
with an external force operator, which the fused path does not take). The
fused integrate path evaluates these in the CUDA kernels; the torch bodies
serve one-shot ``Operator.__call__``.
"""

from typing import Optional

import torch

from ...mesh import FourierMesh
from .._base import CoreGenerator, NonlinearFunc, NonlinearOperator, OperatorLike
from ..generic._convection import _ConvectionCore


class _VorticityConvectionCore(NonlinearFunc):
    def __init__(self) -> None:
        super().__init__()

    def __call__(self, u_fft, f_mesh: FourierMesh, u=None):
        return f_mesh.fft(self.spatial_value(u_fft, f_mesh, u))

    def spatial_value(self, u_fft, f_mesh: FourierMesh, u=None):
        psi = -u_fft * f_mesh.invert_laplacian()
        ux = f_mesh.ifft(f_mesh.grad(1, 1) * psi).real
        uy = f_mesh.ifft(-f_mesh.grad(0, 1) * psi).real
        wx = f_mesh.ifft(f_mesh.grad(0, 1) * u_fft).real
        wy = f_mesh.ifft(f_mesh.grad(1, 1) * u_fft).real
        return ux * wx + uy * wy


class _VorticityConvectionGenerator(CoreGenerator):
    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        if f_mesh.n_dim != 2 or n_channel != 1:
            raise ValueError("Only vorticity in 2Dmesh is supported")
        return _VorticityConvectionCore()


class VorticityConvection(NonlinearOperator):
    """(u . grad) w for a 2D vorticity field."""

    def __init__(self) -> None:
        super().__init__(_VorticityConvectionGenerator())


class _NSPressureConvectionCore(NonlinearFunc):
    def __init__(self, external_force: Optional[OperatorLike] = None) -> None:
        super().__init__(dealiasing_swtich=external_force is None)
        self.external_force = external_force
        self._convection = _ConvectionCore()

    def __call__(self, u_fft, f_mesh: FourierMesh, u=None):
        force = None
        if self.external_force is not None:
            force = self.external_force(u_fft=u_fft, mesh=f_mesh, return_in_fourier=True)
            u_fft = u_fft * f_mesh.low_pass_filter()
            u = f_mesh.ifft(u_fft).real
        elif u is None:
            u = f_mesh.ifft(u_fft).real
        conv = self._convection(u_fft, f_mesh, u)
        if force is not None:
            conv = conv - force
        nv = f_mesh.nabla_vector(1)
        p = f_mesh.invert_laplacian() * torch.sum(nv * conv, dim=1, keepdim=True)
        out = nv * p - conv
        return out + force if force is not None else out


class NSPressureConvection(NonlinearOperator):
    """-grad p - (u . grad) u (+ f) for the velocity form of Navier-Stokes."""

    def __init__(self, external_force: Optional[OperatorLike] = None) -> None:
        super().__init__(_NSPressureConvectionCore(external_force))
