"""Navier-Stokes nonlinear terms (operator/dedicated/_navier_stokes.py).

VorticityConvection: u . grad(w) with u = (d_y psi, -d_x psi), psi = -w/lap
(2D scalar vorticity). NSPressureConvection: -grad p - (u . grad) u with the
pressure from the Leray projection p = lap^-1 div((u . grad) u) (optionally
with an external force operator, which the fused path does not take). The
fused integrate path evaluates these in the CUDA kernels; the torch bodies
serve one-shot ``Operator.__call__``. Vorticity2Velocity, Vorticity2Pressure and
Velocity2Pressure (_navier_stokes.py:75-213) change the channel count and are
post-processing only (one-shot evaluation with torch on the input's device).
"""

from typing import Optional

import torch

from ...mesh import FourierMesh
from .._base import CoreGenerator, LinearCoef, LinearOperator, NonlinearFunc, NonlinearOperator, OperatorLike
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


class _Vorticity2VelocityCore(LinearCoef):
    """-lap^-1 (d_y, -d_x): 2D velocity [u, v] from the vorticity (2 channels from 1)."""

    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        nx, ny = f_mesh.mesh_info[0][-1], f_mesh.mesh_info[1][-1]
        return -1 * f_mesh.invert_laplacian() * torch.cat(
            [f_mesh.grad(1, 1).repeat([1, 1, nx, 1]), -f_mesh.grad(0, 1).repeat([1, 1, 1, ny])], dim=1)


class _Vorticity2VelocityGenerator(CoreGenerator):
    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        if f_mesh.n_dim != 2 or n_channel != 1:
            raise ValueError("Only vorticity in 2Dmesh is supported")
        return _Vorticity2VelocityCore()


class Vorticity2Velocity(LinearOperator):
    """[u, v] = [-d_y lap^-1 w, d_x lap^-1 w] of a 2D vorticity field."""

    def __init__(self) -> None:
        super().__init__(_Vorticity2VelocityGenerator())


def _pressure_from_convection(conv, f_mesh: FourierMesh):
    """p = -lap^-1 div(conv)."""
    div = torch.sum(f_mesh.nabla_vector(1) * conv, dim=1, keepdim=True)
    return -1 * div * f_mesh.invert_laplacian()


class _Vorticity2PressureCore(NonlinearFunc):
    """Pressure of a 2D vorticity field: velocity from the vorticity, then -lap^-1 div((u.grad)u - f)."""

    def __init__(self, external_force: Optional[OperatorLike] = None) -> None:
        super().__init__(dealiasing_swtich=external_force is None)
        self.external_force = external_force
        self._vorticity2velocity = _Vorticity2VelocityCore()
        self._convection = _ConvectionCore()

    def __call__(self, u_fft, f_mesh: FourierMesh, u=None):
        velocity_fft = u_fft * self._vorticity2velocity(f_mesh, 1)
        if self.external_force is not None:
            velocity_fft = velocity_fft * f_mesh.low_pass_filter()
        conv = self._convection(velocity_fft, f_mesh, f_mesh.ifft(velocity_fft).real)
        if self.external_force is not None:
            conv = conv - self.external_force(u_fft=u_fft, mesh=f_mesh, return_in_fourier=True)
        return _pressure_from_convection(conv, f_mesh)


class _Vorticity2PressureGenerator(CoreGenerator):
    def __init__(self, external_force: Optional[OperatorLike] = None) -> None:
        self.external_force = external_force

    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        if f_mesh.n_dim != 2 or n_channel != 1:
            raise ValueError("Only vorticity in 2Dmesh is supported")
        return _Vorticity2PressureCore(self.external_force)


class Vorticity2Pressure(NonlinearOperator):
    """Pressure of a 2D vorticity field."""

    def __init__(self, external_force: Optional[OperatorLike] = None) -> None:
        super().__init__(_Vorticity2PressureGenerator(external_force))


class _Velocity2PressureCore(NonlinearFunc):
    """-lap^-1 div((u.grad)u - f) of a velocity field."""

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
        return _pressure_from_convection(conv, f_mesh)


class Velocity2Pressure(NonlinearOperator):
    """Pressure of a velocity field."""

    def __init__(self, external_force: Optional[OperatorLike] = None) -> None:
        super().__init__(_Velocity2PressureCore(external_force))
