"""GB300-native Fourier-spectral ETD time stepping with the torchfsm API.

``torchfsm_gb300`` keeps the reference's user interface (MeshGrid, the
Operator algebra, ``pde`` constructors, ``Operator.integrate`` with
trajectory recorders) and runs the time stepping in hand-written sm_103a
CUDA kernels behind a C ABI (include/torchfsm_gb300.h).
"""

from . import functional, integrator, mesh, operator, pde, traj_recorder, utils
from .mesh import FourierMesh, MeshGrid
# the reference's package root re-exports its operator package (torchfsm/__init__.py)
from .operator import (Biharmonic, ConservativeConvection, Convection, CoreGenerator, Curl, Div, ExplicitSource,
                       Grad, ImplicitSource, KSConvection, Laplacian, LinearCoef, LinearOperator, NonlinearFunc,
                       NonlinearOperator, NSPressureConvection, Operator, OperatorLike, SpatialDerivative,
                       SpatialTensor, Velocity2Pressure, Vorticity2Pressure, Vorticity2Velocity, VorticityConvection,
                       check_value_with_mesh, default, run_operators)

__version__ = "0.1.0"
