"""The seeded workload fields have the distributions the workloads name (CPU).

2D vorticity: Gaussian random field with shell spectrum E(k) ~ k^4 exp(-(k/4)^2), zero mean, unit
RMS; 3D velocity: E(k) ~ k^2 exp(-(k/3)^2); serving and gradient workloads: band-limited N(0,1)
Fourier series on |k| <= kmax, scaled to an RMS. Same seed, same field; different seeds differ.
"""

import numpy as np
import pytest

from torchfsm_gb300 import initial


def _shell_spectrum(u):
    """Energy per integer shell of the last d axes, averaged over the leading axes."""
    shape = u.shape[2:]
    uh = np.fft.fftn(u, axes=tuple(range(2, u.ndim))) / np.prod(shape)
    power = (np.abs(uh) ** 2).mean(axis=(0, 1))
    _, kmag = initial._integer_wavenumbers(shape)
    shell = np.rint(kmag).astype(int)
    return np.bincount(shell.ravel(), weights=power.ravel())


def test_vorticity_field_moments_and_spectrum():
    w = initial.gaussian_random_field((256, 256), 8, 1, initial.vorticity_spectrum, seed=2024)
    assert w.shape == (8, 1, 256, 256)
    assert np.abs(w.mean(axis=(2, 3))).max() < 1e-12
    assert np.allclose(np.sqrt((w ** 2).mean(axis=(2, 3))), 1.0)
    e = _shell_spectrum(w)
    k = np.arange(2, 13)
    ratio = e[k] / initial.vorticity_spectrum(k.astype(float))
    assert ratio.std() / ratio.mean() < 0.2  # shells 2..12 follow k^4 exp(-(k/4)^2)
    assert e[40:].sum() < 1e-6 * e.sum()     # and nothing far beyond the peak


def test_velocity_field_spectrum_3d():
    u = initial.gaussian_random_field((32, 32, 32), 1, 3, initial.velocity_spectrum, seed=7)
    assert u.shape == (1, 3, 32, 32, 32)
    e = _shell_spectrum(u)
    k = np.arange(2, 8)
    ratio = e[k] / initial.velocity_spectrum(k.astype(float))
    assert ratio.std() / ratio.mean() < 0.25


@pytest.mark.parametrize("shape,kmax,rms", [((1024,), 8, 1.0), ((64, 64), 8, 0.25), ((128, 128), 6, 1.0)])
def test_band_limited_fields(shape, kmax, rms):
    u = initial.band_limited(shape, 4, 2, kmax, seed=11, rms=rms)
    assert np.allclose(np.sqrt((u ** 2).mean(axis=tuple(range(2, u.ndim)))), rms)
    uh = np.fft.fftn(u, axes=tuple(range(2, u.ndim)))
    _, kmag = initial._integer_wavenumbers(shape)
    assert np.abs(uh[..., kmag > kmax]).max() < 1e-9 * np.abs(uh).max()


def test_seeds():
    a = initial.band_limited((64,), 2, 1, 8, seed=3)
    assert np.array_equal(a, initial.band_limited((64,), 2, 1, 8, seed=3))
    assert not np.allclose(a, initial.band_limited((64,), 2, 1, 8, seed=4))
    g = initial.gaussian_random_field((32, 32), 2, 1, initial.vorticity_spectrum, seed=1)
    assert not np.allclose(g[0], g[1])  # samples of one call differ
