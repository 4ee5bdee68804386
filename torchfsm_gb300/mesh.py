"""Meshes and spectral symbols with the reference's interface (torchfsm/mesh.py).

``MeshGrid`` builds coordinates for initial conditions, ``FourierMesh`` the
wavenumbers, derivative symbols, dealias masks and (full complex) transforms
over the last d axes. The fused integrate path takes from here only the
mesh description and the per-axis dealias masks; its transforms and
symbols live in the CUDA library.
"""

from __future__ import annotations

from functools import lru_cache
from typing import Optional, Sequence, Tuple, Union

import numpy as np
import torch

from ._type import FourierTensor, SpatialTensor, ValueList  # noqa: F401
from .utils import default, format_device_dtype

MeshInfo = Sequence[Tuple[float, float, int]]


class MeshGrid:
    """Coordinates of a regular periodic grid (mesh.py:9-145).

    ``mesh_info`` is a sequence of (start, end, n_points). As in the
    reference, coordinate i of an axis is (end - start) * i / n: the start
    offset is not added.
    """

    def __init__(self, mesh_info: MeshInfo, device=None, dtype=None) -> None:
        for axis in mesh_info:
            if len(axis) != 3:
                raise ValueError("each dimension should be a tuple of (start,end,n_points)")
        self.mesh_info = mesh_info
        self.device, self.dtype = format_device_dtype(device, dtype)
        self.n_dim = len(mesh_info)
        self._axes = [None] * self.n_dim
        self._dim_names = ["x", "y", "z"]

    def __len__(self):
        return self.n_dim

    def __getitem__(self, idx: int) -> torch.Tensor:
        if idx >= self.n_dim:
            name = self._dim_names[idx] if idx < 3 else f"id{idx}"
            raise ValueError(f"{name} dim is not defined")
        if self._axes[idx] is None:
            start, end, n = self.mesh_info[idx]
            self._axes[idx] = (end - start) * torch.arange(0, n, device=self.device, dtype=self.dtype) / n
        return self._axes[idx]

    @property
    def x(self):
        return self[0]

    @property
    def y(self):
        return self[1]

    @property
    def z(self):
        return self[2]

    def mesh_grid(self, numpy: bool = False):
        axes = [self[i] for i in range(self.n_dim)]
        if numpy:
            grids = np.meshgrid(*[a.cpu().numpy() for a in axes], indexing="ij")
        else:
            grids = torch.meshgrid(*axes, indexing="ij")
        return grids[0] if len(grids) == 1 else list(grids)

    def bc_mesh_grid(self, batch_size: int = 1, n_channels: int = 1, numpy: bool = False):
        grids = self.mesh_grid()
        if not isinstance(grids, (list, tuple)):
            grids = [grids]
        out = [g.reshape(1, 1, *g.shape).repeat(batch_size, n_channels, *([1] * g.dim())) for g in grids]
        if numpy:
            out = [g.cpu().numpy() for g in out]
        return out[0] if len(out) == 1 else out

    def to(self, device=None, dtype=None):
        self.__init__(self.mesh_info, device=device, dtype=dtype)


class FFTFrequency:
    """Per-axis frequencies fftfreq(n, (end-start)/n) in cycles per unit length (mesh.py:148-216)."""

    def __init__(self, mesh_info: MeshInfo = (), device=None, dtype=None) -> None:
        self.mesh_info = mesh_info
        self.device, self.dtype = format_device_dtype(device, dtype)
        self._fs = [None] * len(mesh_info)
        self._dim_names = ["x", "y", "z"]

    def __len__(self):
        return len(self.mesh_info)

    def __getitem__(self, idx: int) -> torch.Tensor:
        if idx >= len(self):
            raise ValueError(f"fft frequency with id{idx} is not defined")
        if self._fs[idx] is None:
            start, end, n = self.mesh_info[idx]
            self._fs[idx] = torch.fft.fftfreq(n, (end - start) / n, device=self.device, dtype=self.dtype)
        return self._fs[idx]

    @property
    def f_x(self):
        return self[0]

    @property
    def f_y(self):
        return self[1]

    @property
    def f_z(self):
        return self[2]

    def to(self, device=None, dtype=None):
        self.__init__(self.mesh_info, device=device, dtype=dtype)


class BroadcastedFFTFrequency:
    """Frequencies reshaped to broadcast against [B, C, n1, .., nd] (mesh.py:219-291)."""

    def __init__(self, fft_frequency: FFTFrequency) -> None:
        self.fft_frequency = fft_frequency
        self.mesh_shape = tuple(int(m[-1]) for m in fft_frequency.mesh_info)
        self._bks = [None] * len(fft_frequency)
        self._bf_vector = None
        self._dim_names = fft_frequency._dim_names

    def __len__(self):
        return len(self.fft_frequency)

    def __getitem__(self, idx: int) -> torch.Tensor:
        if idx >= len(self):
            raise ValueError(f"fft frequency with id{idx} is not defined")
        if self._bks[idx] is None:
            shape = [1] * (len(self) + 2)
            shape[idx + 2] = self.fft_frequency[idx].shape[0]
            self._bks[idx] = self.fft_frequency[idx].reshape(*shape)
        return self._bks[idx]

    @property
    def bf_vector(self) -> torch.Tensor:
        """[1, d, n1, .., nd]: component i is the axis-i frequency repeated over the grid."""
        if self._bf_vector is None:
            full = (1, 1) + self.mesh_shape
            self._bf_vector = torch.cat([self[i].expand(full) for i in range(len(self))], dim=1).contiguous()
        return self._bf_vector

    @property
    def bf_x(self):
        return self[0]

    @property
    def bf_y(self):
        return self[1]

    @property
    def bf_z(self):
        return self[2]

    def to(self, device=None, dtype=None):
        self.fft_frequency.to(device=device, dtype=dtype)
        self.__init__(self.fft_frequency)


class FourierMesh:
    """Spectral description of a periodic mesh (mesh.py:294-505).

    Symbols are complex tensors broadcastable to [B, C, n1, .., nd]:
    ``grad(i, p) = (2 pi i f_i)^p``, ``laplacian = sum_i grad(i, 2)``,
    ``invert_laplacian`` = 1/laplacian with 1 where the Laplacian is 0,
    ``low_pass_filter(rate)`` = prod_i [|f_i| <= rate * max|f_i|].
    """

    def __init__(self, mesh: Union[MeshInfo, MeshGrid], device=None, dtype=None) -> None:
        if isinstance(mesh, MeshGrid):
            self.mesh_info = mesh.mesh_info
            self.device, self.dtype = format_device_dtype(default(device, mesh.device), default(dtype, mesh.dtype))
        else:
            self.mesh_info = mesh
            self.device, self.dtype = format_device_dtype(device, dtype)
        self.f = FFTFrequency(self.mesh_info, device=self.device, dtype=self.dtype)
        self.bf = BroadcastedFFTFrequency(self.f)
        self.n_dim = len(self.mesh_info)
        self.fft_dim = tuple(-(i + 1) for i in range(self.n_dim))
        self._default_rel_freq_threshold = 2 / 3

    @property
    def mesh_shape(self) -> Tuple[int, ...]:
        return tuple(int(m[2]) for m in self.mesh_info)

    def set_default_rel_freq_threshold(self, threshold: float):
        self._default_rel_freq_threshold = threshold
        self.low_pass_filter.cache_clear()

    @property
    def f_x(self):
        return self.f.f_x

    @property
    def f_y(self):
        return self.f.f_y

    @property
    def f_z(self):
        return self.f.f_z

    @property
    def bf_x(self):
        return self.bf.bf_x

    @property
    def bf_y(self):
        return self.bf.bf_y

    @property
    def bf_z(self):
        return self.bf.bf_z

    @property
    def bf_vector(self):
        return self.bf.bf_vector

    @lru_cache()
    def grad(self, dim_i: int, order: int) -> torch.Tensor:
        return (2j * torch.pi * self.bf[dim_i]) ** order

    @lru_cache()
    def laplacian(self) -> torch.Tensor:
        return self.nabla(2)

    @lru_cache()
    def invert_laplacian(self) -> torch.Tensor:
        lap = self.laplacian()
        return torch.where(lap == 0, 1.0, 1 / lap)

    @lru_cache()
    def nabla(self, order: int = 1) -> torch.Tensor:
        out = self.grad(0, order)
        for i in range(1, self.n_dim):
            out = out + self.grad(i, order)
        return out

    @lru_cache()
    def invert_nabla(self, order: int = 1) -> torch.Tensor:
        nab = self.nabla(order)
        return torch.where(nab == 0, 1.0, 1 / nab)

    @lru_cache()
    def nabla_vector(self, order: int) -> torch.Tensor:
        return (2j * torch.pi * self.bf.bf_vector) ** order

    def axis_keep(self, rel_freq_threshold: Optional[float] = None):
        """Per-axis dealias keep flags [|f_i| <= rate * max|f_i|] in fftfreq order, computed
        in the mesh dtype exactly as ``low_pass_filter`` does."""
        rate = default(rel_freq_threshold, self._default_rel_freq_threshold)
        out = []
        for i in range(self.n_dim):
            a = self.f[i].abs()
            out.append(torch.where(a > a.max() * rate, 0, 1).to(torch.uint8).cpu())
        return out

    @lru_cache()
    def low_pass_filter(self, rel_freq_threshold: Optional[float] = None) -> torch.Tensor:
        rate = default(rel_freq_threshold, self._default_rel_freq_threshold)
        mask = torch.ones((1, 1) + self.mesh_shape, device=self.device, dtype=self.dtype)
        for i in range(self.n_dim):
            a = self.bf[i].abs()
            mask = mask * torch.where(a > a.max() * rate, 0, 1)
        return mask.to(device=self.device, dtype=self.dtype)

    @lru_cache()
    def abs_low_pass_filter(self, abs_freq_threshold: int) -> torch.Tensor:
        mask = torch.ones((1, 1) + self.mesh_shape, device=self.device, dtype=self.dtype)
        for i in range(self.n_dim):
            mask = mask * torch.where(self.bf[i].abs() > abs_freq_threshold, 0, 1)
        return mask.to(device=self.device, dtype=self.dtype)

    def fft(self, u: torch.Tensor) -> torch.Tensor:
        """Full complex spectrum over the last d axes (unnormalised)."""
        return torch.fft.fftn(u, dim=self.fft_dim)

    def ifft(self, u_fft: torch.Tensor) -> torch.Tensor:
        """Inverse of ``fft`` (1/N normalisation); take ``.real`` for a real field."""
        return torch.fft.ifftn(u_fft, dim=self.fft_dim)

    def to(self, device=None, dtype=None):
        self.__init__(self.mesh_info, device=device, dtype=dtype)
        for fn in (self.grad, self.laplacian, self.invert_laplacian, self.nabla, self.invert_nabla,
                   self.nabla_vector, self.low_pass_filter, self.abs_low_pass_filter):
            fn.cache_clear()


def mesh_shape(mesh: Union[MeshInfo, MeshGrid, FourierMesh], batch_size: int = 1, n_channel: int = 1) -> Tuple:
    """(batch, channels, n1, .., nd) of a mesh (mesh.py:507-527)."""
    if isinstance(mesh, (FourierMesh, MeshGrid)):
        mesh = mesh.mesh_info
    return tuple([batch_size, n_channel] + [int(m[2]) for m in mesh])
