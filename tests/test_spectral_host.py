"""Half-spectrum conversions of ``_native.Spectral`` on the CPU (torch arithmetic only).

``half_to_full`` (Hermitian extension) and ``full_to_half`` (the half spectrum of the real part
of ``ifftn(full)``) are the bridge between the library's r2c layout and the reference's full C2C
spectra: the recorders, ``u_0_fft`` inputs, ``return_in_fourier`` outputs and the callback path
all go through them. Checked here against numpy's transforms on 1D, 2D and 3D shapes.
"""

import numpy as np
import pytest
import torch

from torchfsm_gb300._native import Spectral


class _Plan:
    def __init__(self, shape):
        self.shape = tuple(shape)
        self.device = torch.device("cpu")
        self.handle = None


SHAPES = [(16,), (2,), (8, 16), (16, 8), (4, 8, 16), (16, 16, 4)]


def _field(shape, seed, lead=(2, 3)):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(lead + tuple(shape))


@pytest.mark.parametrize("shape", SHAPES)
def test_half_to_full_is_the_full_transform_of_a_real_field(shape):
    u = _field(shape, 1)
    axes = tuple(range(-len(shape), 0))
    half = torch.from_numpy(np.fft.rfftn(u, axes=axes))
    full = Spectral(_Plan(shape)).half_to_full(half)
    np.testing.assert_allclose(full.numpy(), np.fft.fftn(u, axes=axes), rtol=0, atol=1e-10)


@pytest.mark.parametrize("shape", SHAPES)
def test_full_to_half_keeps_what_the_real_part_sees(shape):
    rng = np.random.default_rng(2)
    axes = tuple(range(-len(shape), 0))
    full = rng.standard_normal((2, 3) + tuple(shape)) + 1j * rng.standard_normal((2, 3) + tuple(shape))
    sp = Spectral(_Plan(shape))
    half = sp.full_to_half(torch.from_numpy(full))
    assert half.dtype == torch.complex64
    want = np.fft.rfftn(np.fft.ifftn(full, axes=axes).real, axes=axes)
    np.testing.assert_allclose(half.numpy(), want, rtol=0, atol=1e-5 * np.abs(want).max())
    # and back: the Hermitian extension of that half spectrum is the transform of the real part
    back = sp.half_to_full(half.to(torch.complex128))
    np.testing.assert_allclose(back.numpy(), np.fft.fftn(np.fft.ifftn(full, axes=axes).real, axes=axes), rtol=0,
                               atol=1e-5 * np.abs(want).max())
