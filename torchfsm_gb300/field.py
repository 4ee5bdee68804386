"""Initial-condition and forcing helpers with the reference's names (torchfsm/field.py).

The seeded workloads of this package draw their fields with numpy generators (``initial``).
These helpers keep the reference's API and its torch random draws -- the same calls with the
same shapes, dtypes and devices in the same order -- so that after the same
``torch.manual_seed`` they return the reference's fields:

* ``diffused_noise`` (field.py:8-61): Gaussian noise smoothed by one unit step of
  ``diffusion_coef * Laplacian()`` through ``integrate`` (so, like every ``integrate`` here, it
  needs a CUDA device), then centred and scaled;
* ``truncated_fourier_series`` (field.py:63-125): uniform random amplitudes and phases on every
  mode, kept where each |f_i| is at most ``freq_threshold``, inverse transform, centred and scaled;
* ``kolm_force`` (field.py:128-148): the Kolmogorov forcing operator ``a u - k cos(k l x)``;
* ``wave_1d`` (field.py:151-207): a sum of sines with random wavenumbers, amplitudes and shifts
  plus a random offset.
"""

from __future__ import annotations

import math
from typing import Sequence, Tuple, Union

import torch

from .mesh import FourierMesh, MeshGrid, mesh_shape
from .operator import ExplicitSource, ImplicitSource, Laplacian, Operator

MeshLike = Union[Sequence[Tuple[float, float, int]], MeshGrid, FourierMesh]


def _device_dtype(mesh: MeshLike, device, dtype):
    if isinstance(mesh, (MeshGrid, FourierMesh)):
        device = mesh.device if device is None else device
        dtype = mesh.dtype if dtype is None else dtype
    return device, dtype


def _normalise(u: torch.Tensor, zero_centered: bool, unit_variance: bool, unit_magnitude: bool) -> torch.Tensor:
    """Per sample: subtract the mean, divide by the standard deviation or by the largest |value|."""
    dims = list(range(1, u.dim()))
    if zero_centered:
        u = u - u.mean(dim=dims, keepdim=True)
    if unit_variance:
        u = u / u.std(dim=dims, keepdim=True)
    if unit_magnitude:
        peak = u.abs().reshape(u.shape[0], -1).max(dim=1).values
        u = u / peak.reshape([u.shape[0]] + [1] * (u.dim() - 1))
    return u


def diffused_noise(mesh: MeshLike, diffusion_coef: float = 1.0, zero_centered: bool = True,
                   unit_variance: bool = False, unit_magnitude: bool = True, device=None, dtype=None,
                   batch_size: int = 1, n_channel: int = 1) -> torch.Tensor:
    """Standard normal noise [B, C, n..] after one step of dt = 1 of ``diffusion_coef * Laplacian()``
    (integrated by the library on the noise's device), then normalised per sample."""
    if unit_magnitude and unit_variance:
        raise ValueError("unit_magnitude and unit_variance are mutually exclusive.")
    device, dtype = _device_dtype(mesh, device, dtype)
    u0 = torch.randn(*mesh_shape(mesh, batch_size=batch_size, n_channel=n_channel), device=device, dtype=dtype)
    u = (diffusion_coef * Laplacian()).integrate(u0, dt=1, step=1, mesh=mesh)
    return _normalise(u, zero_centered, unit_variance, unit_magnitude)


def truncated_fourier_series(mesh: MeshLike, freq_threshold: int = 5,
                             amplitude_range: Tuple[float, float] = (-1.0, 1.0),
                             angle_range: Tuple[float, float] = (0.0, 2.0 * math.pi), zero_centered: bool = True,
                             unit_variance: bool = False, unit_magnitude: bool = True, device=None, dtype=None,
                             batch_size: int = 1, n_channel: int = 1) -> torch.Tensor:
    """Real part of the inverse transform of random modes a e^{i phi} (a uniform in
    ``amplitude_range``, phi uniform in ``angle_range``) kept where every |f_i| <= freq_threshold,
    normalised per sample."""
    if unit_magnitude and unit_variance:
        raise ValueError("Cannot set both unit_magnitude and unit_variance to True.")
    device, dtype = _device_dtype(mesh, device, dtype)
    f_mesh = mesh if isinstance(mesh, FourierMesh) else FourierMesh(mesh, device=device, dtype=dtype)
    shape = mesh_shape(f_mesh, batch_size=batch_size, n_channel=n_channel)
    lo, hi = amplitude_range
    amplitude = torch.rand(*shape, device=device, dtype=dtype) * (hi - lo) + lo
    lo, hi = angle_range
    phase = torch.rand(*shape, device=device, dtype=dtype) * (hi - lo) + lo
    modes = amplitude * torch.exp(1j * phase) * f_mesh.abs_low_pass_filter(freq_threshold)
    f_mesh.abs_low_pass_filter.cache_clear()
    u = f_mesh.ifft(modes).real
    return _normalise(u, zero_centered, unit_variance, unit_magnitude)


def kolm_force(x: torch.Tensor, drag_coef: float = -0.1, k: float = 4.0, length_scale: float = 1.0) -> Operator:
    """The Kolmogorov flow forcing of the vorticity equation, a u - k cos(k l x), as an operator:
    ``drag_coef * ImplicitSource()`` (a linear term) minus the explicit source k cos(k l x)."""
    return drag_coef * ImplicitSource() - ExplicitSource(k * torch.cos(k * length_scale * x))


def wave_1d(x: torch.Tensor, min_k: int = 1, max_k: int = 5, min_amplitude: float = 0.5, max_amplitude: float = 1.0,
            n_polynomial: int = 5, zero_mean: bool = False, mean_shift_coef: float = 0.3,
            batched: bool = False) -> torch.Tensor:
    """sum_i a_i sin(k_i (2 pi x / max(x) + s_i)) with integer k_i in [min_k, max_k], a_i uniform in
    [min_amplitude, max_amplitude], s_i uniform in [0, 2 pi), plus (unless ``zero_mean``) a random
    offset per sample; ``x`` is [C, n..] or, with ``batched``, [B, C, n..]."""
    xs = x / x.max() * math.pi * 2
    y = torch.zeros_like(x)
    if not batched:
        xs, y = xs.unsqueeze(0), y.unsqueeze(0)
    batch = xs.shape[0]
    shape = [batch, n_polynomial] + [1] * (xs.dim() - 2)
    k = torch.randint(min_k, max_k + 1, shape, device=x.device, dtype=x.dtype)
    amplitude = torch.rand(*shape, device=x.device, dtype=x.dtype) * (max_amplitude - min_amplitude) + min_amplitude
    shift = torch.rand(*shape, device=x.device, dtype=x.dtype) * math.pi * 2
    for i in range(n_polynomial):
        y = y + amplitude[:, i : i + 1] * torch.sin(k[:, i : i + 1] * (xs + shift[:, i : i + 1]))
    if not zero_mean:
        offset = torch.rand([batch] + [1] * (xs.dim() - 1), device=x.device, dtype=x.dtype)
        y = y + ((offset - 0.5) * 2 * (max_amplitude - min_amplitude) * mean_shift_coef + min_amplitude)
    return y if batched else y.squeeze(0)
