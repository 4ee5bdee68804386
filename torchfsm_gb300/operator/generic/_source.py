"""ImplicitSource: a u (unit form) or f(u) (operator/generic/_source.py:20-74)."""

from typing import Callable, Optional

import torch

from ...mesh import FourierMesh
from .._base import NonlinearFunc, Operator
from ._linear import _ImplicitUnitSourceCore


class _ImplicitFuncSourceCore(NonlinearFunc):
    """fft(f(u)) of a Python callable f; no fused kernel: integrate steps it through the callable."""

    def __init__(self, source_func: Callable[[torch.Tensor], torch.Tensor], non_linear: bool = True) -> None:
        super().__init__(non_linear)
        self.source_func = source_func

    def __call__(self, u_fft, f_mesh: FourierMesh, u=None):
        if u is None:
            u = f_mesh.ifft(u_fft).real
        return f_mesh.fft(self.source_func(u))


class ImplicitSource(Operator):
    """f(u) as a source term; without ``source_func`` the linear identity term u."""

    def __init__(self, source_func: Optional[Callable[[torch.Tensor], torch.Tensor]] = None,
                 non_linear: bool = True) -> None:
        if source_func is None:
            generator = lambda f_mesh, n_channel: _ImplicitUnitSourceCore()
        else:
            generator = lambda f_mesh, n_channel: _ImplicitFuncSourceCore(source_func, non_linear)
        super().__init__(generator)
