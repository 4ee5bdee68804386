"""Large batches run in parts on forked streams (csrc/fsm_api.cu, integrate_impl): the parts'
results equal the same samples integrated alone, and the launch count follows the split."""

import numpy as np
import pytest
import torch

from torchfsm_gb300 import initial, pde

pytestmark = pytest.mark.gpu


def _plan_and_state(batch, n=256):
    dev = torch.device("cuda", 0)
    w = initial.gaussian_random_field((n, n), batch, 1, initial.vorticity_spectrum, 5).astype(np.float32)
    u = torch.tensor(w, device=dev)
    op = pde.NavierStokesVorticity(1000.0)
    mesh = [(0.0, 2 * np.pi, n)] * 2
    op.integrate(u_0=u, mesh=mesh, dt=1e-3, step=1)
    integ = op._state_dict["integrator"]
    return integ.plan, integ.spectral.to_half(u).contiguous()


def test_split_batch_matches_parts_run_alone():
    plan, st0 = _plan_and_state(64)
    whole = st0.clone()
    plan.integrate_half(whole, 6)  # 64 x 256^2: split into parts
    for p0 in range(0, 64, 16):  # 16 samples: one sequence
        part = st0[p0:p0 + 16].clone()
        plan.integrate_half(part, 6)
        assert torch.equal(part, whole[p0:p0 + 16])


def test_launch_count_follows_the_split():
    plan, _ = _plan_and_state(2)
    one = 1 + 10 * 4 * 2  # prime + steps x stages x (row + column)
    assert plan.launch_count(10, 0) == one
    assert plan.launch_count(10, 16) == one
    assert plan.launch_count(10, 64) == 8 * one
