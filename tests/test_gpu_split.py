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


def _unsplit(plan, state, steps):
    """The profiled integrate, which always runs one launch sequence."""
    import ctypes

    from torchfsm_gb300 import _lib

    ws = torch.empty(plan.workspace_bytes(state.shape[0], steps), dtype=torch.uint8, device=state.device)
    ms = (ctypes.c_double * 4)()
    cnt = (ctypes.c_int64 * 4)()
    stream = torch.cuda.current_stream(state.device).cuda_stream
    _lib.check(_lib.load().fsm_integrate_profiled(plan.handle, state.shape[0], ctypes.c_void_p(state.data_ptr()), steps,
                                                  ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel()),
                                                  ctypes.c_void_p(stream), ms, cnt))
    torch.cuda.synchronize()


def test_split_with_per_sample_tables_matches_one_sequence():
    # batched viscosity: one coefficient-table entry per sample, offset per part
    dev = torch.device("cuda", 0)
    B, n = 48, 256
    nu = torch.linspace(0.005, 0.02, B, dtype=torch.float64, device=dev).reshape(B, 1, 1, 1)
    op = pde.Burgers(nu)
    w = initial.band_limited((n, n), B, 2, 6, 9, 0.25).astype(np.float32)
    u = torch.tensor(w, device=dev)
    op.integrate(u_0=u, mesh=[(0.0, 2 * np.pi, n)] * 2, dt=0.01, step=1)
    integ = op._state_dict["integrator"]
    assert integ.plan.launch_count(1, B) > integ.plan.launch_count(1, 0)  # this batch splits
    st0 = integ.spectral.to_half(u).contiguous()
    a, b = st0.clone(), st0.clone()
    integ.plan.integrate_half(a, 5)
    _unsplit(integ.plan, b, 5)
    assert torch.equal(a, b)


def test_split_recording_matches_unrecorded_runs():
    plan, st0 = _plan_and_state(64)
    steps = 6
    traj = torch.empty((64, 4) + tuple(st0.shape[1:]), dtype=torch.complex64, device=st0.device)
    rec = st0.clone()
    slots = [0, -1, 1, -1, 2, -1, 3]  # frames at steps 0, 2, 4, 6
    plan.integrate_half(rec, steps, slots=slots, traj=traj)
    for frame, k in enumerate((0, 2, 4, 6)):
        ref = st0.clone()
        if k:
            plan.integrate_half(ref, k)
        assert torch.equal(traj[:, frame], ref), f"frame at step {k}"
    assert torch.equal(traj[:, 3], rec)
