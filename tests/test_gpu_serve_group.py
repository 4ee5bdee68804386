"""Serving groups (fsm_serve_group_*): engines of different grid sizes ticked together. The 1D KS
engines of every size advance in ONE launch per tick (k_line_multi); 2D engines of square grids
in one launch per pass (k_axis0_multi2 / k_plane_row_multi); other mixes tick in lockstep.
Each request's result equals a plain integration of its samples, and served KS solves match the
reference's FP64 runs (golden fixtures)."""

import os

import numpy as np
import pytest
import torch

import cases as C
from oracle import spectral as S
from torchfsm_gb300 import _lib, _native, initial, serving
from torchfsm_gb300.mesh import FourierMesh

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda", 0)
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _engine(kind, n, capacity, chunk, stream, graphs=True):
    op, mesh, C_ = serving.problem(kind, n)
    f_mesh = FourierMesh(mesh, device=DEV, dtype=torch.float32)
    op.register_mesh(f_mesh, C_)
    prog = _native.lower(op._linear_terms, op._nonlinear_funcs, f_mesh, C_, op._de_aliasing_rate)
    L = op._linear_coef64(DEV)
    with torch.cuda.stream(stream):
        plan = _native.NativePlan(prog, 0.05, _lib.FSM_SETDRK4, DEV, linear_coef64=L, table_batch=capacity)
    torch.cuda.synchronize()
    pool = _native.ServePool(plan, capacity, chunk, stream, graphs=graphs)
    return prog, L, plan, pool


def _half(plan, kind, n, batch, seed, field=None):
    shape = (n,) if kind == "ks1d" else (n, n)
    if field is None:
        field = initial.band_limited(shape, batch, plan.n_channel, 8, seed, 1.0 if kind == "ks1d" else 0.25)
    h = _native.Spectral(plan).to_half(torch.tensor(field, dtype=torch.float32, device=DEV)).contiguous()
    torch.cuda.synchronize()
    return h


def _plain(prog, L, half, steps, dt):
    plan = _native.NativePlan(prog, dt, _lib.FSM_SETDRK4, DEV, linear_coef64=L)
    st = half.clone()
    plan.integrate_half(st, steps)
    torch.cuda.synchronize()
    return st


def _drain(group, pools):
    done = {id(p): [] for p in pools}
    for _ in range(100000):
        group.tick()
        busy = group.poll(wait=True)
        for p in pools:
            ids, _ = p.poll(False)
            done[id(p)] += ids
        if not busy and all(p.stats()["occupied"] == 0 and p.stats()["waiting"] == 0 for p in pools):
            torch.cuda.synchronize()
            return done
    raise AssertionError("the group did not drain")


def _rel(a, b):
    return float((a - b).abs().pow(2).sum().sqrt() / b.abs().pow(2).sum().sqrt())


def test_line_group_one_launch_per_tick_matches_plain_integration():
    """KS 1D at 256, 1024 and 4096 points: every tick is one kernel launch over all three sizes,
    and every request ends where a plain integration of its samples with its own dt ends."""
    stream = torch.cuda.Stream(DEV)
    sizes = (256, 1024, 4096)
    eng = {n: _engine("ks1d", n, capacity=9, chunk=16, stream=stream) for n in sizes}
    group = _native.ServeGroup([eng[n][3] for n in sizes], tick_ms=0.0)
    specs = {256: [(0, 3, 40, 0.05), (1, 9, 23, 0.03), (2, 2, 7, 0.08)],
             1024: [(10, 1, 31, 0.02), (11, 4, 12, 0.06)],
             4096: [(20, 2, 19, 0.02), (21, 5, 9, 0.01)]}
    halves, refs = {}, {}
    for n in sizes:
        prog, L, plan, pool = eng[n]
        for rid, b, steps, dt in specs[n]:
            halves[rid] = _half(plan, "ks1d", n, b, 300 + rid)
            refs[rid] = _plain(prog, L, halves[rid], steps, dt)
            pool.submit(rid, steps, dt, halves[rid])
    done = _drain(group, [eng[n][3] for n in sizes])
    for n in sizes:
        assert sorted(done[id(eng[n][3])]) == sorted(r[0] for r in specs[n])
    for rid in halves:
        assert _rel(halves[rid], refs[rid]) <= 1e-6, rid
    st = group.stats()
    assert st["one_launch"] == 1 and st["ticks"] > 0 and st["launches"] == st["ticks"]
    group.close()
    for n in sizes:
        eng[n][3].__del__()


def test_line_group_serves_reference_fp64_solutions():
    """The reference's FP64 KS runs at 1024 and 4096 points (golden fixtures, 200 steps) served
    through one group, beside requests of another size in the same ticks."""
    stream = torch.cuda.Stream(DEV)
    names = ("ks1d_n1024", "ks1d_n4096")
    pools, halves = [], {}
    for rid, name in enumerate(names):
        case = C._case(name)
        n = case["mesh"][0][2]
        _, _, plan, pool = _engine("ks1d", n, capacity=4, chunk=32, stream=stream)
        halves[rid] = _half(plan, "ks1d", n, case["batch"], 0, field=C.initial_condition(name))
        pool.submit(rid, case["step"], case["dt"], halves[rid])
        pools.append((pool, plan))
    _, _, plan5, pool5 = _engine("ks1d", 512, capacity=4, chunk=32, stream=stream)
    pool5.submit(99, 150, 0.05, _half(plan5, "ks1d", 512, 4, 7))
    group = _native.ServeGroup([p for p, _ in pools] + [pool5], tick_ms=0.0)
    _drain(group, [p for p, _ in pools] + [pool5])
    for rid, name in enumerate(names):
        g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
        out = _native.Spectral(pools[rid][1]).to_physical(halves[rid]).cpu().numpy().astype(np.float64)
        ref = g["final_kept"].astype(np.float64)
        err = max(S.rel_l2(out[k], ref[i]) for i, k in enumerate(g["keep"]))
        print(f"{name} served: rel-L2 {err:.2e}")
        assert err <= 1e-5, name
    group.close()
    for p, _ in pools:
        p.__del__()
    pool5.__del__()


def test_group_2d_one_launch_per_pass_matches_plain_integration():
    """2D Burgers at 64^2 and 128^2 advanced by one group: each column and row pass of a tick is one
    launch over both sizes (a priming pass, then two launches per stage)."""
    stream = torch.cuda.Stream(DEV)
    eng = {n: _engine("burgers2d", n, capacity=6, chunk=8, stream=stream) for n in (64, 128)}
    group = _native.ServeGroup([eng[n][3] for n in (64, 128)], tick_ms=0.0)
    specs = {64: [(0, 2, 20, 0.05), (1, 3, 11, 0.03)], 128: [(10, 4, 14, 0.02), (11, 1, 6, 0.07)]}
    halves, refs = {}, {}
    for n, rows in specs.items():
        prog, L, plan, pool = eng[n]
        for rid, b, steps, dt in rows:
            halves[rid] = _half(plan, "burgers2d", n, b, 500 + rid)
            refs[rid] = _plain(prog, L, halves[rid], steps, dt)
            pool.submit(rid, steps, dt, halves[rid])
    _drain(group, [eng[n][3] for n in (64, 128)])
    for rid in halves:
        assert _rel(halves[rid], refs[rid]) <= 1e-6, rid
    st = group.stats()
    assert st["one_launch"] == 0 and st["one_launch_per_pass"] == 1
    # every tick: one priming launch and 2 launches per stage of each of its k steps
    assert st["launches"] > st["ticks"] and (st["launches"] - st["ticks"]) % 8 == 0
    group.close()


def test_group_of_mixed_kinds_ticks_in_lockstep():
    """A 1D KS engine and a 2D Burgers engine in one group: no shared kernel, so the members launch one
    after the other in each tick; results are unchanged."""
    stream = torch.cuda.Stream(DEV)
    ks = _engine("ks1d", 256, capacity=4, chunk=8, stream=stream)
    bg = _engine("burgers2d", 64, capacity=4, chunk=8, stream=stream)
    group = _native.ServeGroup([ks[3], bg[3]], tick_ms=0.0)
    halves, refs = {}, {}
    for rid, (eng, kind, n, b, steps, dt) in enumerate([(ks, "ks1d", 256, 3, 17, 0.05),
                                                        (bg, "burgers2d", 64, 2, 13, 0.03)]):
        prog, L, plan, pool = eng
        halves[rid] = _half(plan, kind, n, b, 700 + rid)
        refs[rid] = _plain(prog, L, halves[rid], steps, dt)
        pool.submit(rid, steps, dt, halves[rid])
    _drain(group, [ks[3], bg[3]])
    for rid in halves:
        assert _rel(halves[rid], refs[rid]) <= 1e-6, rid
    st = group.stats()
    assert st["one_launch"] == 0 and st["one_launch_per_pass"] == 0
    group.close()


def test_group_refusals():
    stream = torch.cuda.Stream(DEV)
    a = _engine("ks1d", 256, 2, 4, stream)[3]
    b = _engine("ks1d", 512, 2, 4, stream)[3]
    other = _engine("ks1d", 1024, 2, 4, torch.cuda.Stream(DEV))[3]
    with pytest.raises(_lib.FsmError):
        _native.ServeGroup([a, other])  # engines on different streams
    with pytest.raises(_lib.FsmError):
        _native.ServeGroup([a, a])  # listed twice
    group = _native.ServeGroup([a, b])
    with pytest.raises(_lib.FsmError):
        a.tick()  # a member is ticked through its group
    with pytest.raises(_lib.FsmError):
        _native.ServeGroup([b])  # already grouped
    assert _lib.load().fsm_serve_destroy(a.handle) != 0  # destroying a member first is refused
    group.close()
    assert a.tick() == 0  # released: ticks alone again (nothing queued)


def test_server_groups_the_1d_buckets():
    """The server's 1D KS buckets share one group; results are the same as with per-bucket ticks."""
    reqs = serving.make_stream(12, seed=21, rate_hz=0.0, max_steps=150)
    res = {}
    for grouped in (True, False):
        rq = serving.make_stream(12, seed=21, rate_hz=0.0, max_steps=150)
        srv = serving.SolveServer(DEV, hbm_budget_bytes=2 << 30, chunk=16, group_lines=grouped)
        srv.run(rq, realtime=False)
        for r in rq:
            r._copied.synchronize()
        res[grouped] = {r.rid: r.result.clone() for r in rq}
        if grouped:
            assert len(srv.groups) == (1 if len({r.n for r in reqs if r.kind == "ks1d"}) > 1 else 0)
        srv.close()
    for rid in res[True]:
        assert _rel(res[True][rid], res[False][rid]) <= 1e-6, rid
