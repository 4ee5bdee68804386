from ._ks_convection import KSConvection
from ._navier_stokes import NSPressureConvection, VorticityConvection
