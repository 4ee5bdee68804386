"""Seeded initial-condition generators for the benchmark workloads.

Plain numpy (PCG64), so that the same seed gives bit-identical fields on any
host; the fields are then handed to torch. These generators are not part of
the reference (its ``field.py`` draws with torch's global RNG); they produce
the synthetic inputs of the named workloads:

* ``gaussian_random_field``: random phases with a prescribed shell energy
  spectrum E(k), zero mean, unit RMS (2D vorticity: E ~ k^4 exp(-(k/4)^2);
  3D velocity: E ~ k^2 exp(-(k/3)^2)).
* ``band_limited``: a random Fourier series with N(0,1) complex coefficients
  on the integer modes |k| <= kmax, then scaled to a given RMS.
"""

from __future__ import annotations

from typing import Callable, Sequence, Tuple

import numpy as np


def _integer_wavenumbers(shape: Sequence[int]):
    ks = [np.fft.fftfreq(n, d=1.0 / n) for n in shape]
    grids = np.meshgrid(*ks, indexing="ij")
    kmag = np.sqrt(sum(g * g for g in grids))
    return grids, kmag


def gaussian_random_field(
    shape: Sequence[int],
    batch: int,
    channels: int,
    spectrum: Callable[[np.ndarray], np.ndarray],
    seed: int,
    rms: float = 1.0,
) -> np.ndarray:
    """Real field [batch, channels, *shape] (float64) with shell spectrum ``spectrum(|k|)``.

    The per-mode amplitude is sqrt(E(k) / k^(d-1)) so that the shell-summed
    energy follows E(k); phases are uniform. Each (sample, channel) is
    shifted to zero mean and scaled to the given RMS.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    d = len(shape)
    _, kmag = _integer_wavenumbers(shape)
    with np.errstate(divide="ignore", invalid="ignore"):
        amp = np.sqrt(np.where(kmag > 0, spectrum(kmag) / np.maximum(kmag, 1e-300) ** (d - 1), 0.0))
    out = np.empty((batch, channels) + tuple(shape), dtype=np.float64)
    for b in range(batch):
        for c in range(channels):
            phase = rng.uniform(0.0, 2.0 * np.pi, size=tuple(shape))
            coef = amp * np.exp(1j * phase)
            f = np.fft.ifftn(coef).real
            f = f - f.mean()
            s = np.sqrt(np.mean(f * f))
            out[b, c] = f * (rms / s if s > 0 else 0.0)
    return out


def band_limited(
    shape: Sequence[int],
    batch: int,
    channels: int,
    kmax: float,
    seed: int,
    rms: float = 1.0,
) -> np.ndarray:
    """Real field [batch, channels, *shape] from N(0,1) complex modes with |k| <= kmax.

    The real part of the inverse transform is taken, the mean is kept (the
    k = 0 mode is one of the drawn modes), and each (sample, channel) is
    scaled to the given RMS.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    _, kmag = _integer_wavenumbers(shape)
    keep = kmag <= kmax
    out = np.empty((batch, channels) + tuple(shape), dtype=np.float64)
    for b in range(batch):
        for c in range(channels):
            coef = (rng.standard_normal(tuple(shape)) + 1j * rng.standard_normal(tuple(shape))) * keep
            f = np.fft.ifftn(coef).real
            s = np.sqrt(np.mean(f * f))
            out[b, c] = f * (rms / s if s > 0 else 0.0)
    return out


def vorticity_spectrum(k: np.ndarray) -> np.ndarray:
    """E(k) ~ k^4 exp(-(k/4)^2)."""
    return k ** 4 * np.exp(-((k / 4.0) ** 2))


def velocity_spectrum(k: np.ndarray) -> np.ndarray:
    """E(k) ~ k^2 exp(-(k/3)^2)."""
    return k ** 2 * np.exp(-((k / 3.0) ** 2))


def mesh_points(mesh_info: Sequence[Tuple[float, float, int]]):
    """Coordinates (end - start) * i / N per axis, start ignored as in the reference's MeshGrid."""
    return [(e - s) * np.arange(n, dtype=np.float64) / n for (s, e, n) in mesh_info]
