"""Coefficient tables built on the GPU (FP64, rounded to FP32) against the reference's FP64 tables.

The library stores the exponential tables as exp(dt L) - 1 and exp(dt L / 2) - 1 (its kernels form
exp(dt L) u as u + (E - 1) u), so those two are compared with the reference's E - 1 and E2 - 1."""

import os

import numpy as np
import pytest
import torch

from torchfsm_gb300 import _lib, _native
from torchfsm_gb300.mesh import FourierMesh

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
pytestmark = pytest.mark.gpu

MESHES = {"ks1d": [(0, 32 * np.pi, 64)], "ns2d": [(0, 2 * np.pi, 32)] * 2, "kdv1d": [(0, 20.0, 64)]}


@pytest.mark.parametrize("tag", sorted(MESHES))
@pytest.mark.parametrize("m,r", [(16, 1.0), (32, 2.0), (6, 1.5)])
def test_setdrk4_tables_match_reference(tag, m, r):
    g = np.load(os.path.join(GOLDEN, "phi_coefs.npz"))
    mesh = MESHES[tag]
    h = mesh[-1][2] // 2 + 1
    L = torch.tensor(g[f"{tag}_L"]).reshape((1, 1) + tuple(n for _, _, n in mesh))
    dt = float(g[f"{tag}_dt"])
    prog = _native.SpectralProgram(tuple(mesh), 1, keep=FourierMesh(mesh).axis_keep(2 / 3))
    plan = _native.NativePlan(prog, dt, _lib.FSM_SETDRK4, torch.device("cuda"), n_integration_points=m,
                              integration_radius=r, linear_coef64=L.to("cuda"))
    tabs = plan.tables().cpu().numpy()
    if (m, r) in ((16, 1.0), (32, 2.0)):
        refs = [g[f"{tag}_m{m}_{k}"] for k in ("E", "E2", "c1", "c4", "c5", "c6")]
    else:
        from oracle import spectral as S

        t = S.setdrk_coefs(4, g[f"{tag}_L"], dt, m, r)
        refs = [t[k] for k in ("E", "E2", "c1", "c4", "c5", "c6")]
    for i, ref in enumerate(refs):
        if i < 2:
            ref = np.asarray(ref) - 1.0
        ref_half = np.broadcast_to(ref, L.shape)[..., :h].reshape(-1)
        got = tabs[i]
        scale = np.abs(ref_half).max()
        np.testing.assert_allclose(got, ref_half, rtol=2e-6, atol=2e-7 * scale, err_msg=f"{tag} table {i}")
