"""Vector-calculus cores: Grad, Div, Curl (operator/generic/_grad.py, _div.py, _curl.py).

They serve one-shot ``Operator.__call__`` / ``functional`` evaluation (post-processing) with
torch spectral multiplies on the input's device. ``integrate`` of Grad (a linear term that
changes the channel count) reports it unsupported; Div and Curl are nonlinear terms without a
fused kernel, so ``integrate`` steps them through the callback path, where their values
broadcast against the state as in the reference's stage arithmetic.
"""

import torch

from ...mesh import FourierMesh
from .._base import CoreGenerator, LinearCoef, LinearOperator, NonlinearFunc, NonlinearOperator


class _GradCore(LinearCoef):
    """2 pi i f_i for every axis: [1, d, n1..] (applied to a scalar field)."""

    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        return f_mesh.nabla_vector(1)


class _GradGenerator(CoreGenerator):
    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        if n_channel != 1:
            raise ValueError("The Grad operator only supports scalar field.")
        return _GradCore()


class Grad(LinearOperator):
    """Spatial gradient of a scalar field."""

    def __init__(self) -> None:
        super().__init__(_GradGenerator())


class _DivCore(NonlinearFunc):
    """sum_i 2 pi i f_i u_i (no dealiasing)."""

    def __init__(self) -> None:
        super().__init__(False)

    def __call__(self, u_fft, f_mesh: FourierMesh, u=None):
        return torch.sum(f_mesh.nabla_vector(1) * u_fft, dim=1, keepdim=True)


class _DivGenerator(CoreGenerator):
    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        if f_mesh.n_dim != n_channel:
            raise ValueError("div operator only works for vector field with the same dimension as mesh")
        return _DivCore()


class Div(NonlinearOperator):
    """Divergence of a vector field with as many components as mesh axes."""

    def __init__(self) -> None:
        super().__init__(_DivGenerator())


class _Curl2DCore(NonlinearFunc):
    """d_x u_y - d_y u_x."""

    def __init__(self) -> None:
        super().__init__(False)

    def __call__(self, u_fft, f_mesh: FourierMesh, u=None):
        return f_mesh.grad(0, 1) * u_fft[:, 1:2] - f_mesh.grad(1, 1) * u_fft[:, 0:1]


class _Curl3DCore(NonlinearFunc):
    """(d_y u_z - d_z u_y, d_z u_x - d_x u_z, d_x u_y - d_y u_x)."""

    def __init__(self) -> None:
        super().__init__(False)

    def __call__(self, u_fft, f_mesh: FourierMesh, u=None):
        g = [f_mesh.grad(i, 1) for i in range(3)]
        return torch.cat([g[1] * u_fft[:, 2:3] - g[2] * u_fft[:, 1:2],
                          g[2] * u_fft[:, 0:1] - g[0] * u_fft[:, 2:3],
                          g[0] * u_fft[:, 1:2] - g[1] * u_fft[:, 0:1]], dim=1)


class _CurlGenerator(CoreGenerator):
    def __call__(self, f_mesh: FourierMesh, n_channel: int):
        if f_mesh.n_dim != n_channel:
            raise ValueError("div operator only works for vector field with the same dimension as mesh")
        if n_channel > 3 or n_channel < 2:
            raise ValueError("div operator only works for 2D or 3D vector field")
        return _Curl2DCore() if n_channel == 2 else _Curl3DCore()


class Curl(NonlinearOperator):
    """Curl of a 2D (scalar result) or 3D (vector result) vector field."""

    def __init__(self) -> None:
        super().__init__(_CurlGenerator())
