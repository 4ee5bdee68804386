"""PDE constructors with the reference's names and coefficients (torchfsm/pde.py:13-100)."""

from typing import Optional

from .operator import (
    Biharmonic,
    Convection,
    KSConvection,
    Laplacian,
    NSPressureConvection,
    Operator,
    SpatialDerivative,
    VorticityConvection,
)


def Burgers(nu: float) -> Operator:
    """u_t = -u . grad u + nu lap u."""
    return nu * Laplacian() - Convection()


def KuramotoSivashinsky() -> Operator:
    """1D: phi_t = -phi_xx - phi_xxxx - phi phi_x (1D meshes only)."""
    op = -Laplacian() - Biharmonic() - Convection()
    op.register_additional_check(lambda dim_value, dim_mesh: dim_value == 1 and dim_mesh == 1)
    return op


def KuramotoSivashinskyHighDim() -> Operator:
    """phi_t = -lap phi - lap^2 phi - 0.5 |grad phi|^2."""
    return -Laplacian() - Biharmonic() - KSConvection()


def KortewegDeVries(dispersion_coef=1, convection_coef: float = 6.0) -> Operator:
    """phi_t = -c1 phi_xxx + c2 phi phi_x."""
    return -dispersion_coef * SpatialDerivative(0, 3) + convection_coef * Convection()


def NavierStokesVorticity(Re: float, force: Optional[Operator] = None) -> Operator:
    """w_t + (u . grad) w = lap w / Re (+ force, the curl of the body force)."""
    op = -VorticityConvection() + 1 / Re * Laplacian()
    if force is not None:
        op += force
    return op


def NavierStokes(Re: float, force: Optional[Operator] = None) -> Operator:
    """u_t = -grad p - (u . grad) u + lap u / Re (+ f)."""
    return NSPressureConvection(force) + 1 / Re * Laplacian()
