from ._convection import ConservativeConvection, Convection
from ._linear import Biharmonic, Laplacian, SpatialDerivative
from ._source import ImplicitSource
from ._vector import Curl, Div, Grad
