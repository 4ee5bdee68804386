"""Function forms of the operators (torchfsm/functional.py): one-shot evaluation of an
operator on a field, ``f(u=None, u_fft=None, mesh=...)`` returning the physical result.

Each function builds the operator and calls it once (``Operator.__call__``): programs
the library lowers run through the fused kernels, the channel-changing ones through
torch spectral multiplies on the field's device.
"""

from typing import Optional, Sequence, Tuple, Union

import torch

from .mesh import FourierMesh, MeshGrid
from .operator import (Biharmonic, ConservativeConvection, Convection, Curl, Div, Grad, KSConvection, Laplacian,
                       OperatorLike, SpatialDerivative, Vorticity2Velocity, VorticityConvection)

MeshLike = Union[Sequence[Tuple[float, float, int]], MeshGrid, FourierMesh]


def biharmonic(u: Optional[torch.Tensor] = None, u_fft: Optional[torch.Tensor] = None,
               mesh: Optional[MeshLike] = None) -> torch.Tensor:
    """functional.py:9-28."""
    return Biharmonic()(u=u, u_fft=u_fft, mesh=mesh)


def conservative_convection(u: Optional[torch.Tensor] = None, u_fft: Optional[torch.Tensor] = None,
                            mesh: Optional[MeshLike] = None) -> torch.Tensor:
    """functional.py:31-50."""
    return ConservativeConvection()(u=u, u_fft=u_fft, mesh=mesh)


def convection(u: Optional[torch.Tensor] = None, u_fft: Optional[torch.Tensor] = None,
               mesh: Optional[MeshLike] = None) -> torch.Tensor:
    """functional.py:53-73."""
    return Convection()(u=u, u_fft=u_fft, mesh=mesh)


def curl(u: Optional[torch.Tensor] = None, u_fft: Optional[torch.Tensor] = None,
         mesh: Optional[MeshLike] = None) -> torch.Tensor:
    """functional.py:76-96."""
    return Curl()(u=u, u_fft=u_fft, mesh=mesh)


def div(u: Optional[torch.Tensor] = None, u_fft: Optional[torch.Tensor] = None,
        mesh: Optional[MeshLike] = None) -> torch.Tensor:
    """functional.py:99-119."""
    return Div()(u=u, u_fft=u_fft, mesh=mesh)


def grad(u: Optional[torch.Tensor] = None, u_fft: Optional[torch.Tensor] = None,
         mesh: Optional[MeshLike] = None) -> torch.Tensor:
    """functional.py:122-142."""
    return Grad()(u=u, u_fft=u_fft, mesh=mesh)


def laplacian(u: Optional[torch.Tensor] = None, u_fft: Optional[torch.Tensor] = None,
              mesh: Optional[MeshLike] = None) -> torch.Tensor:
    """functional.py:145-164."""
    return Laplacian()(u=u, u_fft=u_fft, mesh=mesh)


def spatial_derivative(dim_index: int, order: int, u: Optional[torch.Tensor] = None,
                       u_fft: Optional[torch.Tensor] = None, mesh: Optional[MeshLike] = None) -> torch.Tensor:
    """functional.py:167-190."""
    return SpatialDerivative(dim_index, order)(u=u, u_fft=u_fft, mesh=mesh)


def ks_convection(u: Optional[torch.Tensor] = None, u_fft: Optional[torch.Tensor] = None,
                  mesh: Optional[MeshLike] = None, remove_mean: bool = True) -> torch.Tensor:
    """functional.py:193-214."""
    return KSConvection(remove_mean)(u=u, u_fft=u_fft, mesh=mesh)


def vorticity_convection(u: Optional[torch.Tensor] = None, u_fft: Optional[torch.Tensor] = None,
                         mesh: Optional[MeshLike] = None) -> torch.Tensor:
    """functional.py:216-236."""
    return VorticityConvection()(u=u, u_fft=u_fft, mesh=mesh)


def _get_fft_with_mesh(value: Optional[torch.Tensor] = None, value_fft: Optional[torch.Tensor] = None,
                       mesh: Optional[MeshLike] = None):
    """The spectrum of a field and its FourierMesh (functional.py:238-267)."""
    if value_fft is None:
        f_mesh = mesh if isinstance(mesh, FourierMesh) else FourierMesh(mesh, device=value.device, dtype=value.dtype)
        value_fft = f_mesh.fft(value)
    else:
        f_mesh = mesh if isinstance(mesh, FourierMesh) else FourierMesh(mesh, device=value_fft.device,
                                                                        dtype=value_fft.dtype)
    return value_fft, f_mesh


def vorticity2velocity(vorticity: Optional[torch.Tensor] = None, vorticity_fft: Optional[torch.Tensor] = None,
                       mesh: Optional[MeshLike] = None) -> torch.Tensor:
    """functional.py:270-290."""
    return Vorticity2Velocity()(u=vorticity, u_fft=vorticity_fft, mesh=mesh)


def velocity2pressure(velocity: Optional[torch.Tensor] = None, velocity_fft: Optional[torch.Tensor] = None,
                      mesh: Optional[MeshLike] = None, external_force: Optional[OperatorLike] = None) -> torch.Tensor:
    """-lap^-1 div((u.grad)u - f) (functional.py:293-324)."""
    velocity_fft, f_mesh = _get_fft_with_mesh(value=velocity, value_fft=velocity_fft, mesh=mesh)
    conv = Convection()(u_fft=velocity_fft, mesh=f_mesh, return_in_fourier=True)
    if external_force is not None:
        conv = conv - external_force(u_fft=velocity_fft, mesh=f_mesh, return_in_fourier=True)
    conv = Div()(u_fft=conv, mesh=f_mesh, return_in_fourier=True)
    return Laplacian().solve(b_fft=-1 * conv, mesh=f_mesh, n_channel=1)


def vorticity2pressure(vorticity: Optional[torch.Tensor] = None, vorticity_fft: Optional[torch.Tensor] = None,
                       mesh: Optional[MeshLike] = None, external_force: Optional[OperatorLike] = None) -> torch.Tensor:
    """Velocity from the vorticity, then velocity2pressure (functional.py:327-361)."""
    vorticity_fft, f_mesh = _get_fft_with_mesh(value=vorticity, value_fft=vorticity_fft, mesh=mesh)
    velocity_fft = Vorticity2Velocity()(u_fft=vorticity_fft, mesh=f_mesh, return_in_fourier=True)
    conv = Convection()(u_fft=velocity_fft, mesh=f_mesh, return_in_fourier=True)
    if external_force is not None:  # the force takes the vorticity spectrum (functional.py:350-353)
        conv = conv - external_force(u_fft=vorticity_fft, mesh=f_mesh, return_in_fourier=True)
    conv = Div()(u_fft=conv, mesh=f_mesh, return_in_fourier=True)
    return Laplacian().solve(b_fft=-1 * conv, mesh=f_mesh, n_channel=1)
