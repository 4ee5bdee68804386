"""Host-side checks of the serving request stream (no GPU)."""

import numpy as np

from torchfsm_gb300 import serving


def test_stream_requests_do_not_depend_on_the_arrival_rate():
    # latency in the mix is compared request by request with the one-at-a-time run of the
    # burst stream, so both streams must hold the same requests
    burst = serving.make_stream(24, seed=11, rate_hz=0.0)
    timed = serving.make_stream(24, seed=11, rate_hz=8.0)
    for a, b in zip(burst, timed):
        assert (a.kind, a.n, a.batch, a.steps, a.dt) == (b.kind, b.n, b.batch, b.steps, b.dt)
        assert np.array_equal(a.u0.numpy(), b.u0.numpy())
        assert a.arrival == 0.0
    arr = [r.arrival for r in timed]
    assert all(x < y for x, y in zip(arr, arr[1:]))
    # mean gap near 1 / rate
    assert 0.05 < arr[-1] / len(arr) < 0.25


def test_stream_mix_covers_both_kinds_and_ranges():
    reqs = serving.make_stream(200, seed=3, rate_hz=0.0)
    kinds = {(r.kind, r.n) for r in reqs}
    assert {("ks1d", n) for n in (256, 512, 1024, 2048, 4096)} <= kinds
    assert {("burgers2d", n) for n in (64, 128, 256)} <= kinds
    assert all(1 <= r.batch <= 32 and 100 <= r.steps <= 2000 and 0.01 <= r.dt <= 0.1 for r in reqs)


def test_request_reports_a_diverged_result():
    import torch

    from torchfsm_gb300.serving import SolveRequest

    r = SolveRequest(0, "ks1d", 8, 1, 10, 0.1, torch.zeros(1, 1, 8))
    assert r.finite is None  # no result yet
    r.result = torch.ones(1, 1, 8)
    assert r.finite is None  # copy to the host not yet complete
    r.t_done = 1.0
    assert r.finite is True
    r.result[0, 0, 3] = float("nan")
    assert r.finite is False
    r.result[0, 0, 3] = float("inf")
    assert r.finite is False
