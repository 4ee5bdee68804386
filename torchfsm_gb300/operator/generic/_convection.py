"""(u . grad) u and div(u u) (operator/generic/_convection.py, _conservative_convection.py).

The fused integrate path evaluates these in the CUDA kernels; the torch
bodies here serve one-shot ``Operator.__call__``.
"""

from ...mesh import FourierMesh
from .._base import CoreGenerator, NonlinearFunc, NonlinearOperator


class _ConvectionCore(NonlinearFunc):
    """sum_i u_i d_i u_c for a vector field with as many channels as dimensions."""

    def __init__(self):
        super().__init__()

    def __call__(self, u_fft, f_mesh: FourierMesh, u=None):
        return f_mesh.fft(self.spatial_value(u_fft, f_mesh, u))

    def spatial_value(self, u_fft, f_mesh: FourierMesh, u=None):
        if u is None:
            u = f_mesh.ifft(u_fft).real
        grads = f_mesh.ifft(f_mesh.nabla_vector(1).unsqueeze(2) * u_fft.unsqueeze(1)).real  # [B, d, C, ..]
        return (u.unsqueeze(2) * grads).sum(1)


class _ConvectionGenerator(CoreGenerator):
    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        if f_mesh.n_dim != n_channel:
            raise ValueError("convection operator only works for vector field with the same dimension as mesh")
        return _ConvectionCore()


class Convection(NonlinearOperator):
    """(u . grad) u."""

    def __init__(self) -> None:
        super().__init__(_ConvectionGenerator())


class _ConservativeConvectionCore(NonlinearFunc):
    """sum_i d_i (u_i u_c)."""

    def __init__(self):
        super().__init__()

    def __call__(self, u_fft, f_mesh: FourierMesh, u=None):
        if u is None:
            u = f_mesh.ifft(u_fft).real
        uu_fft = f_mesh.fft(u.unsqueeze(2) * u.unsqueeze(1))
        return (f_mesh.nabla_vector(1).unsqueeze(2) * uu_fft).sum(1)


class _ConservativeConvectionGenerator(CoreGenerator):
    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        if f_mesh.n_dim != n_channel:
            raise ValueError("div operator only works for vector field with the same dimension as mesh")
        return _ConservativeConvectionCore()


class ConservativeConvection(NonlinearOperator):
    """div(u u)."""

    def __init__(self) -> None:
        super().__init__(_ConservativeConvectionGenerator())
