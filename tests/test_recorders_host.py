"""Recorders, spectral inputs and outputs of ``Operator.integrate`` on the CPU.

The recorders are fed by the same integrate driver on every path: blocks of half spectra
written by the library (AutoRecorder, CPURecorder) or the per-step ``record(step, frame)``
protocol on full spectra (DiskRecorder, RandomBatchWisedRecorder, user subclasses). These
tests drive them through ``integrate`` of a program stepped through its Python callables, with
the CPU stand-ins of ``tests/cpu_library.py`` for the library's tables and transforms, and hold
every recorder to the reference's float64 trajectory of the same program (golden vectors) or to
the AutoRecorder trajectory of the same run.
"""

import os

import numpy as np
import pytest
import torch

import cases as C
import cpu_library as CL
from oracle import spectral as S
from torchfsm_gb300 import traj_recorder as TR

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-5
NAME = "allencahn1d_n64"  # 2 samples, 64 points, 100 SETDRK4 steps, frames every 20 steps


@pytest.fixture(autouse=True)
def cpu_library(monkeypatch):
    CL.install(monkeypatch)


def _op():
    M = C.namespace("torchfsm_gb300")
    return C.CALLBACK_CASES[NAME]["build"](M)


def _u0():
    return torch.tensor(C.initial_condition(NAME), dtype=torch.float32)


def _integrate(rec=None, steps=None, **kw):
    case = C.CALLBACK_CASES[NAME]
    return _op().integrate(u_0=kw.pop("u_0", _u0()), mesh=case["mesh"], dt=case["dt"],
                           step=case["step"] if steps is None else steps, trajectory_recorder=rec, **kw)


def _golden_traj():
    return np.load(os.path.join(GOLDEN, f"{NAME}.npz"))["traj"]


def test_interval_controller_matches_the_reference_trajectory():
    out = _integrate(TR.AutoRecorder(TR.IntervalController(interval=20)))
    assert S.rel_l2(out.numpy(), _golden_traj()) <= TOL


def test_interval_controller_start():
    ctl = TR.IntervalController(interval=20, start=40)
    assert [s for s in range(101) if ctl(s)] == [40, 60, 80, 100]
    out = _integrate(TR.AutoRecorder(ctl))
    assert S.rel_l2(out.numpy(), _golden_traj()[:, 2:]) <= TOL


def test_cpu_recorder_and_per_step_subclass_give_the_same_trajectory():
    every20 = TR.IntervalController(interval=20)
    auto = _integrate(TR.AutoRecorder(every20))

    class PerStep(TR.AutoRecorder):  # overriding the hook keeps the per-step protocol
        def _record(self, step, frame):
            super()._record(step, frame)

    per_step = PerStep(every20)
    assert not per_step._accepts_blocks()
    cpu = _integrate(TR.CPURecorder(every20))
    ps = _integrate(per_step)
    assert cpu.device.type == "cpu"
    assert torch.allclose(cpu, auto, rtol=0, atol=1e-6)
    assert S.rel_l2(ps.numpy(), auto.numpy()) <= 1e-6


def test_initial_state_can_be_left_out():
    out = _integrate(TR.AutoRecorder(TR.IntervalController(interval=20), include_initial_state=False))
    assert S.rel_l2(out.numpy(), _golden_traj()[:, 1:]) <= TOL


def test_return_in_fourier_with_and_without_a_recorder():
    spec = _integrate(TR.AutoRecorder(TR.IntervalController(interval=20)), return_in_fourier=True)
    assert spec.is_complex() and spec.shape == _golden_traj().shape
    phys = torch.fft.ifftn(spec, dim=(-1,)).real
    assert S.rel_l2(phys.numpy(), _golden_traj()) <= TOL
    final = _integrate(return_in_fourier=True)
    assert final.is_complex()
    assert S.rel_l2(torch.fft.ifftn(final, dim=(-1,)).real.numpy(), _golden_traj()[:, -1]) <= TOL


def test_spectral_initial_condition():
    u0 = _u0()
    a = _integrate(steps=30)
    b = _integrate(steps=30, u_0=None, u_0_fft=torch.fft.fftn(u0, dim=(-1,)))
    assert S.rel_l2(b.numpy(), a.numpy()) <= 1e-6


def test_zero_steps_return_the_initial_state():
    u0 = _u0()
    out = _integrate(steps=0)
    assert S.rel_l2(out.numpy(), u0.numpy()) <= 1e-6
    traj = _integrate(TR.AutoRecorder(), steps=0)
    assert traj.shape == (2, 1, 1, 64)


@pytest.mark.parametrize("fmt", ["torch", "numpy"])
def test_disk_recorder_chunks_concatenate_to_the_trajectory(tmp_path, fmt):
    every20 = TR.IntervalController(interval=20)
    rec = TR.DiskRecorder(every20, cache_dir=str(tmp_path) + os.sep, cache_freq=2, save_format=fmt)
    assert _integrate(rec) is None
    # 6 frames (steps 0, 20, .., 100) in chunks of 2, named by their last recorded step
    names = sorted(os.listdir(tmp_path), key=lambda n: int(n.split("_")[-1].split(".")[0]))
    assert [n.split(".")[0] for n in names] == ["temp_cache_20", "temp_cache_60", "temp_cache_100"]
    chunks = [torch.load(tmp_path / n) if fmt == "torch" else torch.from_numpy(np.load(tmp_path / n))
              for n in names]
    got = torch.cat(chunks, dim=1)
    assert S.rel_l2(got.numpy(), _golden_traj()) <= TOL


def test_disk_recorder_saves_the_last_short_chunk(tmp_path):
    rec = TR.DiskRecorder(TR.IntervalController(interval=20), cache_dir=str(tmp_path) + os.sep, cache_freq=4)
    _integrate(rec)
    names = sorted(os.listdir(tmp_path))
    assert names == ["temp_cache_100", "temp_cache_60"]
    assert torch.load(tmp_path / "temp_cache_60").shape[1] == 4
    assert torch.load(tmp_path / "temp_cache_100").shape[1] == 2


def test_random_batch_wised_recorder_frames():
    auto = _integrate(TR.AutoRecorder())  # every step: 101 frames
    np.random.seed(7)
    rec = TR.RandomBatchWisedRecorder(simulation_steps=100, recorder_interval=10, n_recorded_frames=3)
    out = _integrate(rec)
    ids = rec._recorded_frame_id
    assert out.shape == (2, 3, 1, 64) and ids.shape == (2, 3)
    for b in range(2):
        assert 1 <= ids[b, 0] and ids[b, -1] < 100
        assert np.all(np.diff(ids[b]) == 10)
        assert S.rel_l2(out[b].numpy(), auto[b, ids[b]].numpy()) <= 1e-6
