"""The library's serving engine (fsm_serve_*) driven directly: each request's result equals a
plain integration of its samples with a plan of its own dt; cancellation of waiting and active
requests; refusals."""

import pytest
import torch

from torchfsm_gb300 import _lib, _native, initial, serving
from torchfsm_gb300.mesh import FourierMesh

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda", 0)


def _setup(kind, n, capacity, chunk, graphs=True, op=None):
    if op is None:
        op, mesh, C = serving.problem(kind, n)
    else:
        _, mesh, C = serving.problem(kind, n)
        C = 1
    f_mesh = FourierMesh(mesh, device=DEV, dtype=torch.float32)
    op.register_mesh(f_mesh, C)
    prog = _native.lower(op._linear_terms, op._nonlinear_funcs, f_mesh, C, op._de_aliasing_rate)
    L = op._linear_coef64(DEV)
    stream = torch.cuda.Stream(DEV)
    with torch.cuda.stream(stream):
        plan = _native.NativePlan(prog, 0.05, _lib.FSM_SETDRK4, DEV, linear_coef64=L, table_batch=capacity)
    torch.cuda.synchronize()
    pool = _native.ServePool(plan, capacity, chunk, stream, graphs=graphs)
    return prog, L, plan, pool


def _half(plan, kind, n, batch, seed):
    shape = (n,) if kind == "ks1d" else (n, n)
    C = plan.n_channel
    u = initial.band_limited(shape, batch, C, 8, seed, 1.0 if kind == "ks1d" else 0.25).astype("float32")
    h = _native.Spectral(plan).to_half(torch.from_numpy(u).to(DEV)).contiguous()
    torch.cuda.synchronize()
    return h


def _reference(prog, L, half, steps, dt):
    plan = _native.NativePlan(prog, dt, _lib.FSM_SETDRK4, DEV, linear_coef64=L)
    st = half.clone()
    plan.integrate_half(st, steps)
    torch.cuda.synchronize()
    return st


def _drain(pool):
    done = []
    for _ in range(10000):
        pool.tick()
        ids, busy = pool.poll(wait=True)
        done += ids
        st = pool.stats()
        if not busy and st["occupied"] == 0 and st["waiting"] == 0:
            torch.cuda.synchronize()
            return done
    raise AssertionError("the engine did not drain")


def _rel(a, b):
    return float((a - b).abs().pow(2).sum().sqrt() / b.abs().pow(2).sum().sqrt())


@pytest.mark.parametrize("kind,n,capacity,chunk,graphs", [
    ("ks1d", 256, 6, 7, True),
    ("burgers2d", 64, 5, 8, True),
    ("burgers2d", 64, 5, 8, False),
])
def test_requests_match_plain_integration(kind, n, capacity, chunk, graphs):
    prog, L, plan, pool = _setup(kind, n, capacity, chunk, graphs)
    specs = [(0, 2, 30, 0.05), (1, 3, 21, 0.03), (2, 2, 9, 0.07), (3, 1, 5, 0.1)]
    halves = {rid: _half(plan, kind, n, b, 100 + rid) for rid, b, _, _ in specs}
    refs = {rid: _reference(prog, L, halves[rid], steps, dt) for rid, _, steps, dt in specs}
    for rid, _, steps, dt in specs:
        pool.submit(rid, steps, dt, halves[rid])
        assert pool.status(rid)[0] == _lib.FSM_SERVE_WAITING
    done = _drain(pool)
    assert sorted(done) == [0, 1, 2, 3]
    for rid, _, _, _ in specs:
        err = _rel(halves[rid], refs[rid])
        assert err <= 1e-6, f"request {rid}: {err:.2e}"
        assert pool.status(rid)[0] == _lib.FSM_SERVE_UNKNOWN
    st = pool.stats()
    assert st["completed"] == 4 and st["active"] == 0 and st["launches"] > 0
    assert (st["graph_replays"] > 0) == graphs or kind == "ks1d"


def test_cancel_waiting_and_active():
    kind, n = "ks1d", 256
    prog, L, plan, pool = _setup(kind, n, capacity=2, chunk=5)
    a = _half(plan, kind, n, 2, 7)
    b = _half(plan, kind, n, 1, 8)
    a0, b0 = a.clone(), b.clone()
    pool.submit(10, 20, 0.05, a)
    pool.submit(11, 10, 0.05, b)
    k = pool.tick()  # admits 10 (both slots); 11 waits
    assert k == 4  # min(chunk 5, 20 steps) rounded down to a power of two for graph replay
    assert pool.status(10) == (_lib.FSM_SERVE_ACTIVE, 20)
    assert pool.status(11) == (_lib.FSM_SERVE_WAITING, 10)
    pool.cancel(11)
    assert pool.status(11)[0] == _lib.FSM_SERVE_UNKNOWN
    pool.cancel(10)  # tick in flight: leaves when it completes
    ids, busy = pool.poll(wait=True)
    torch.cuda.synchronize()
    assert ids == [] and not busy
    assert torch.equal(b, b0)  # never admitted: untouched
    ref = _reference(prog, L, a0, k, 0.05)
    assert _rel(a, ref) <= 1e-6  # the state it reached
    st = pool.stats()
    assert st["cancelled"] == 2 and st["completed"] == 0 and st["occupied"] == 0 and st["waiting"] == 0
    with pytest.raises(_lib.FsmError):
        pool.cancel(10)


def test_refusals():
    kind, n = "ks1d", 256
    prog, L, plan, pool = _setup(kind, n, capacity=3, chunk=4)
    h = _half(plan, kind, n, 4, 1)
    with pytest.raises(_lib.FsmError):
        pool.submit(1, 10, 0.05, h)  # 4 samples > 3 slots
    with pytest.raises(_lib.FsmError):
        pool.submit(2, 10, 0.05, h[:, :, :10].contiguous())  # wrong sample shape
    h2 = _half(plan, kind, n, 1, 2)
    pool.submit(3, 10, 0.05, h2)
    with pytest.raises(_lib.FsmError):
        pool.submit(3, 10, 0.05, h2)  # id pending
    with pytest.raises(_lib.FsmError):
        pool.submit(4, 0, 0.05, h2)  # no steps
    _drain(pool)
    # samples coupled by the batch-wide KS mean cannot share ticks with other requests
    from torchfsm_gb300 import pde

    with pytest.raises(_lib.UnsupportedProgram):
        _setup("burgers2d", 64, 4, 4, op=pde.KuramotoSivashinskyHighDim())
