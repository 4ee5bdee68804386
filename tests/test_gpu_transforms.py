"""GPU transforms (fsm_rfftn / fsm_irfftn) against numpy on the same inputs."""

import math

import numpy as np
import pytest
import torch

from torchfsm_gb300 import _lib, _native
from torchfsm_gb300.mesh import FourierMesh

pytestmark = pytest.mark.gpu


def _spectral(shape):
    mesh = [(0.0, 2 * math.pi, n) for n in shape]
    prog = _native.SpectralProgram(tuple(mesh), 1, keep=FourierMesh(mesh).axis_keep(2 / 3))
    plan = _native.NativePlan(prog, 0.1, _lib.FSM_ETDRK0, torch.device("cuda"))
    return _native.Spectral(plan)


@pytest.mark.parametrize("shape", [(16,), (128,), (1024,), (4096,), (16, 32), (64, 64), (256, 256), (128, 512),
                                   (32, 16, 16)])
def test_rfftn_matches_numpy(shape):
    rng = np.random.default_rng(7)
    x = rng.standard_normal((3,) + shape).astype(np.float32)
    sp = _spectral(shape)
    half = sp.to_half(torch.tensor(x, device="cuda")).cpu().numpy()
    ref = np.fft.rfftn(x.astype(np.float64), axes=tuple(range(1, len(shape) + 1)))
    err = np.linalg.norm(half - ref) / np.linalg.norm(ref)
    assert err < 2e-6, err
    back = sp.to_physical(torch.tensor(half, device="cuda")).cpu().numpy()
    err2 = np.linalg.norm(back - x) / np.linalg.norm(x)
    assert err2 < 2e-6, err2


def test_full_half_round_trip():
    sp = _spectral((32, 64))
    x = torch.randn(2, 1, 32, 64, device="cuda")
    full = torch.fft.fftn(x.double(), dim=(-2, -1))
    half = sp.to_half(x)
    np.testing.assert_allclose(sp.half_to_full(half).cpu().numpy(), full.cpu().numpy(), rtol=0, atol=2e-4)
    np.testing.assert_allclose(sp.full_to_half(full).cpu().numpy(), half.cpu().numpy(), rtol=0, atol=2e-4)
