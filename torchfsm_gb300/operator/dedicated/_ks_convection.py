"""KSConvection: 0.5 |grad phi|^2 (operator/dedicated/_ks_convection.py).

With ``remove_mean`` the mean is taken over the whole tensor, batch
included, as in the reference (_ks_convection.py:35-36).
"""

import torch

from ...mesh import FourierMesh
from .._base import CoreGenerator, NonlinearFunc, NonlinearOperator


class _KSConvectionCore(NonlinearFunc):
    def __init__(self, remove_mean: bool) -> None:
        super().__init__()
        self.remove_mean = remove_mean

    def __call__(self, u_fft, f_mesh: FourierMesh, u=None):
        return f_mesh.fft(self.spatial_value(u_fft, f_mesh, u))

    def spatial_value(self, u_fft, f_mesh: FourierMesh, u=None):
        grad_u = f_mesh.ifft(f_mesh.nabla_vector(1) * u_fft).real
        re = 0.5 * torch.sum(grad_u ** 2, dim=1, keepdim=True)
        return re - re.mean() if self.remove_mean else re


class _KSConvectionGenerator(CoreGenerator):
    def __init__(self, remove_mean: bool) -> None:
        self.remove_mean = remove_mean

    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        if n_channel != 1:
            raise NotImplementedError("KSConvection only supports scalar field")
        return _KSConvectionCore(self.remove_mean)


class KSConvection(NonlinearOperator):
    """0.5 |grad phi|^2 of a scalar field."""

    def __init__(self, remove_mean: bool = True) -> None:
        super().__init__(_KSConvectionGenerator(remove_mean))
