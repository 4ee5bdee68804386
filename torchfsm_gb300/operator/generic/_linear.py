"""Linear cores: Laplacian, Biharmonic, SpatialDerivative, ImplicitSource (unit form).

Symbols follow operator/generic/_laplacian.py:7-15, _biharmonic.py:8-16,
_spatial_derivative.py:7-20 and _source.py:9-17 of the reference.
"""

import torch

from ...mesh import FourierMesh
from .._base import CoreGenerator, LinearCoef, LinearOperator


class _LaplacianCore(LinearCoef):
    """sum_i (2 pi i f_i)^2, repeated over the channels."""

    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        return torch.cat([f_mesh.laplacian()] * n_channel, dim=1)


class Laplacian(LinearOperator):
    """Laplacian of every channel."""

    def __init__(self) -> None:
        super().__init__(_LaplacianCore())


class _BiharmonicCore(LinearCoef):
    """Square of the Laplacian symbol, repeated over the channels."""

    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        lap = f_mesh.laplacian()
        return torch.cat([lap * lap] * n_channel, dim=1)


class Biharmonic(LinearOperator):
    """Biharmonic operator of every channel."""

    def __init__(self) -> None:
        super().__init__(_BiharmonicCore())


class _SpatialDerivativeCore(LinearCoef):
    """(2 pi i f_dim)^order."""

    def __init__(self, dim_index: int, order: int) -> None:
        self.dim_index = dim_index
        self.order = order

    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        return f_mesh.grad(self.dim_index, self.order)


class _SpatialDerivativeGenerator(CoreGenerator):
    def __init__(self, dim_index: int, order: int) -> None:
        self.dim_index = dim_index
        self.order = order

    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        if n_channel != 1:
            raise ValueError("The SpatialDerivative operator only supports scalar field.")
        return _SpatialDerivativeCore(self.dim_index, self.order)


class SpatialDerivative(LinearOperator):
    """d^order / dx_dim^order of a scalar field."""

    def __init__(self, dim_index: int, order: int) -> None:
        super().__init__(_SpatialDerivativeGenerator(dim_index, order))


class _ImplicitUnitSourceCore(LinearCoef):
    """The identity (symbol 1): ``a * ImplicitSource()`` is the linear term a u."""

    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        return torch.ones_like(f_mesh.bf_x)
