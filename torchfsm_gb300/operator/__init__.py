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
from .dedicated import KSConvection, NSPressureConvection, VorticityConvection
from .generic import Biharmonic, ConservativeConvection, Convection, ImplicitSource, Laplacian, SpatialDerivative
