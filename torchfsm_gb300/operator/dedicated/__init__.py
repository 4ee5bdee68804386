from ._ks_convection import KSConvection
from ._navier_stokes import (NSPressureConvection, Velocity2Pressure, Vorticity2Pressure, Vorticity2Velocity,
                             VorticityConvection)
