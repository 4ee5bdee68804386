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
