"""Serving loop: every request's result is the same alone (plain integrate) and in the mix."""

import pytest
import torch

from torchfsm_gb300 import serving

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_the_mix():
    device = torch.device("cuda", 0)
    reqs = serving.make_stream(14, seed=3, rate_hz=0.0, max_steps=150, min_steps=20)
    with serving.SolveServer(device, hbm_budget_bytes=1 << 30, chunk=17) as server:
        server.run(reqs, realtime=False)
    ops = {}
    for r in reqs:
        alone, _ = serving.solve_alone(r, device, ops)
        assert r.result.shape == alone.shape
        err = float((r.result.double() - alone.double()).norm() / alone.double().norm())
        assert err <= 1e-6, f"request {r.rid} ({r.kind} N={r.n} B={r.batch}): {err:.2e}"
        assert torch.isfinite(r.result).all()


def test_threaded_loop_gives_the_same_results():
    device = torch.device("cuda", 0)
    reqs = serving.make_stream(10, seed=4, rate_hz=0.0, max_steps=120, min_steps=20)
    with serving.SolveServer(device, hbm_budget_bytes=1 << 30, chunk=13) as server:
        server.run_threaded(reqs, realtime=False)
    ops = {}
    for r in reqs:
        alone, _ = serving.solve_alone(r, device, ops)
        err = float((r.result.double() - alone.double()).norm() / alone.double().norm())
        assert err <= 1e-6 and r.t_done is not None


def test_admission_respects_capacity_and_compacts():
    device = torch.device("cuda", 0)
    reqs = [r for r in serving.make_stream(40, seed=5, rate_hz=0.0, max_steps=60, min_steps=10) if r.kind == "ks1d"]
    with serving.SolveServer(device, hbm_budget_bytes=1 << 20, chunk=9, max_slots=40) as server:
        server.run(reqs, realtime=False)
        for b in server.buckets.values():
            st = b.engine.stats()
            assert st["occupied"] == 0 and st["waiting"] == 0 and st["active"] == 0 and not b.pending
            assert st["completed"] == sum(1 for r in reqs if (r.kind, r.n) == (b.kind, b.n))
    assert all(r.result is not None and r.t_done >= r.t_admit for r in reqs)


def test_close_releases_engines_before_plans():
    device = torch.device("cuda", 0)
    reqs = serving.make_stream(4, seed=8, rate_hz=0.0, max_steps=40, min_steps=10)
    server = serving.SolveServer(device, hbm_budget_bytes=1 << 28, chunk=8)
    server.run_threaded(reqs, realtime=False)
    buckets = list(server.buckets.values())
    server.close()
    assert server.buckets == {} and all(b.engine is None and b.plan is None for b in buckets)
    assert all(r.result is not None for r in reqs)


def test_graph_replays_match_direct_launches():
    device = torch.device("cuda", 0)
    out = {}
    for graphs in (False, True):
        reqs = serving.make_stream(12, seed=6, rate_hz=0.0, max_steps=90, min_steps=30)
        with serving.SolveServer(device, hbm_budget_bytes=1 << 30, chunk=8, graphs=graphs) as server:
            server.run(reqs, realtime=False)
            out[graphs] = [r.result for r in reqs]
            if graphs:
                assert server.graph_replays > 0
            else:
                assert server.graph_replays == 0
    for a, b in zip(out[False], out[True]):
        assert torch.equal(a, b)
