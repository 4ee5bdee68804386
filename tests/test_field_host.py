"""The initial-condition helpers (torchfsm_gb300.field) against the reference's outputs (CPU).

Each call of ``tests/golden/make_field_golden.py`` runs again here after the same
``torch.manual_seed``: the helpers make the reference's torch random draws in the same order, so
the fields agree to rounding. ``diffused_noise`` integrates its noise with the library (one ETDRK0
step of the Laplacian), which runs here on the CPU stand-ins of ``tests/cpu_library.py``, in FP32
(the reference runs the golden call in float64).
"""

import math
import os

import numpy as np
import pytest
import torch

import cpu_library as CL
import make_field_golden as G
from torchfsm_gb300 import field as F

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "field_helpers.npz")


@pytest.mark.parametrize("name,seed,call", G.CALLS, ids=[c[0] for c in G.CALLS])
def test_helper_matches_reference(name, seed, call, monkeypatch):
    CL.install(monkeypatch)
    ref = np.load(GOLDEN)[name]
    torch.manual_seed(seed)
    got = call(F).numpy()
    assert got.shape == ref.shape
    tol = 1e-5 if name.startswith("diffused") else 1e-12
    assert np.abs(got - ref).max() <= tol * max(1.0, np.abs(ref).max())


def test_exclusive_normalisations():
    with pytest.raises(ValueError):
        F.truncated_fourier_series([(0, 1, 16)], unit_variance=True, unit_magnitude=True)
    with pytest.raises(ValueError):
        F.diffused_noise([(0, 1, 16)], unit_variance=True, unit_magnitude=True)


def test_kolm_force_terms():
    x = torch.arange(32, dtype=torch.float64).reshape(1, 1, 1, 32) / 32 * 2 * math.pi
    op = F.kolm_force(x, drag_coef=-0.2, k=4.0)
    op.register_mesh([(0, 2 * math.pi, 32), (0, 2 * math.pi, 32)], 1)
    (coef, lin), = op._linear_terms
    assert coef == -0.2 and torch.all(lin(op._state_dict["f_mesh"], 1) == 1)
    (ncoef, src), = op._nonlinear_funcs
    assert ncoef == -1 and torch.allclose(src.source_physical, 4.0 * torch.cos(4.0 * x))
