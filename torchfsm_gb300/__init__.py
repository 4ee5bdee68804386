"""GB300-native Fourier-spectral ETD time stepping with the torchfsm API.

``torchfsm_gb300`` keeps the reference's user interface (MeshGrid, the
Operator algebra, ``pde`` constructors, ``Operator.integrate`` with
trajectory recorders) and runs the time stepping in hand-written sm_103a
CUDA kernels behind a C ABI (include/torchfsm_gb300.h).
"""

from . import functional, integrator, mesh, operator, pde, traj_recorder, utils
from .mesh import FourierMesh, MeshGrid
from .operator import Operator

__version__ = "0.1.0"
