"""fsm_integrate_static: the integrate entry point for callers that cannot allocate.

Some callers of this library may not call cudaMalloc (or anything that
allocates) once they are running: host callbacks, plugin hosts that forbid
allocation after start-up, real-time loops. For them fsm_integrate_static
takes its scratch from a fixed device array inside the library instead of a
caller workspace. This test drives it through the C ABI with ctypes and
checks, on two calls in a row, that it gives the same result as
fsm_integrate with a torch-allocated workspace (relative L2 within 1e-5, the
tolerance of the parity tests), and that work larger than the array is
rejected with a clear error. It lives in its own file, collected last, and
passes alone in a fresh process as well as after the other tests.
"""

import ctypes
import math

import pytest
import torch

from torchfsm_gb300 import _lib, initial, pde

pytestmark = pytest.mark.gpu

TOL = 1e-5
N, BATCH, STEPS, DT = 64, 3, 10, 5e-3
MESH = [(0.0, 2 * math.pi, N), (0.0, 2 * math.pi, N)]


def _plan_and_state():
    w0 = initial.gaussian_random_field((N, N), BATCH, 1, initial.vorticity_spectrum, seed=17)
    u = torch.tensor(w0, dtype=torch.float32, device="cuda")
    op = pde.NavierStokesVorticity(1000)
    op.integrate(u_0=u, mesh=MESH, dt=DT, step=1)  # registers the mesh and builds the plan
    integ = op._state_dict["integrator"]
    return op, integ.plan, integ.spectral.to_half(u).contiguous()


def _rel(a, b):
    a = torch.view_as_real(a).double()
    b = torch.view_as_real(b).double()
    return float((a - b).norm() / b.norm())


def test_static_entry_matches_workspace_entry_on_two_calls():
    lib = _lib.load()
    op, plan, state0 = _plan_and_state()
    stream = torch.cuda.current_stream().cuda_stream
    ws_bytes = plan.workspace_bytes(BATCH, STEPS)
    assert ws_bytes <= _lib.FSM_STATIC_SCRATCH_BYTES
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    ref = state0.clone()
    got = state0.clone()
    for call in range(2):
        rc = lib.fsm_integrate(plan.handle, BATCH, ctypes.c_void_p(ref.data_ptr()), STEPS, None, None, 0,
                               ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws_bytes), ctypes.c_void_p(stream))
        assert rc == _lib.FSM_OK, _lib.last_error()
        rc = lib.fsm_integrate_static(plan.handle, BATCH, ctypes.c_void_p(got.data_ptr()), STEPS,
                                      ctypes.c_void_p(stream))
        assert rc == _lib.FSM_OK, _lib.last_error()
        torch.cuda.synchronize()
        err = _rel(got, ref)
        assert err <= TOL, f"call {call}: rel-L2 {err:.3e}"
        assert bool(torch.isfinite(torch.view_as_real(got)).all())


def test_static_entry_allocates_nothing_after_a_warm_up_call():
    """The promise the entry point exists for: after one warm-up call (which loads the kernels
    and backs the array), further calls leave the device's free memory unchanged."""
    lib = _lib.load()
    op, plan, state0 = _plan_and_state()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    got = state0.clone()
    rc = lib.fsm_integrate_static(plan.handle, BATCH, ctypes.c_void_p(got.data_ptr()), STEPS, stream)
    assert rc == _lib.FSM_OK, _lib.last_error()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        rc = lib.fsm_integrate_static(plan.handle, BATCH, ctypes.c_void_p(got.data_ptr()), STEPS, stream)
        assert rc == _lib.FSM_OK, _lib.last_error()
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before, (free_before, free_after)


def test_static_entry_rejects_work_above_the_array():
    lib = _lib.load()
    op, plan, state0 = _plan_and_state()
    big = 1
    while plan.workspace_bytes(big, STEPS) <= _lib.FSM_STATIC_SCRATCH_BYTES:
        big *= 2
    state = torch.zeros((big,) + tuple(state0.shape[1:]), dtype=torch.complex64, device="cuda")
    rc = lib.fsm_integrate_static(plan.handle, big, ctypes.c_void_p(state.data_ptr()), STEPS,
                                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == _lib.FSM_ERR_INVALID
    assert "static limit" in _lib.last_error()
