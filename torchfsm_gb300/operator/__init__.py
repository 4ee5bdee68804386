"""Operators with the reference's names (torchfsm/operator)."""

from ._base import (
    CoreGenerator,
    ExplicitSource,
    LinearCoef,
    LinearOperator,
    NonlinearFunc,
    NonlinearOperator,
    Operator,
    OperatorLike,
    check_value_with_mesh,
)
from .dedicated import (KSConvection, NSPressureConvection, Velocity2Pressure, Vorticity2Pressure, Vorticity2Velocity,
                        VorticityConvection)
from .generic import (Biharmonic, ConservativeConvection, Convection, Curl, Div, Grad, ImplicitSource, Laplacian,
                      SpatialDerivative)
from .._type import SpatialTensor
from ..mesh import FourierMesh, MeshGrid
from ..utils import default


def run_operators(u, operators, mesh):
    """Apply each operator to ``u`` (one forward transform shared by all), lazily: returns a map
    over ``operator(u_fft=..., mesh=...)`` (operator/__init__.py:12-30 of the reference). A mesh
    given as (start, end, n) tuples is built on ``u``'s device and dtype (the reference builds it
    with FourierMesh's defaults, which then fails the device check for CUDA inputs)."""
    if not isinstance(mesh, FourierMesh):
        if isinstance(mesh, MeshGrid):
            mesh = FourierMesh(mesh)
        else:
            mesh = FourierMesh(mesh, device=u.device, dtype=u.dtype)
    u_fft = mesh.fft(u)
    return map(lambda op: op(u_fft=u_fft, mesh=mesh), operators)
