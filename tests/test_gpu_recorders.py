"""The recorder variants on the fused CUDA path (traj_recorder.py:127-264 of the reference).

``CPURecorder`` (the kernels' frames moved to pinned host memory as one block), ``DiskRecorder``
(chunks in torch.save / np.save format) and ``RandomBatchWisedRecorder`` (per-sample random
frame windows, fed through the per-step protocol) drive ``Operator.integrate`` of fused programs
on the GPU -- the 1D line kernel, the 2D plane passes and the 3D volume passes -- and are held to
the reference's float64 trajectories of the same cases (golden vectors), or to the AutoRecorder
trajectory of the same run.
"""

import os

import numpy as np
import pytest
import torch

import cases as C
from oracle import spectral as S
from torchfsm_gb300 import traj_recorder as TR

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-5
pytestmark = pytest.mark.gpu

# fused cases with recorded trajectories: 1D line kernel, 2D plane passes, 3D volume passes
RECORDED = ["ks1d_n128", "ns2d_n32", "nsvel3d_n16"]


def _integrate(name, rec, steps=None, **kw):
    case = C.CASES[name]
    M = C.namespace("torchfsm_gb300")
    op = case["build"](M)
    u0 = torch.tensor(C.initial_condition(name), dtype=torch.float32, device="cuda")
    return op.integrate(u_0=u0, mesh=case["mesh"], dt=case["dt"], step=case["step"] if steps is None else steps,
                        trajectory_recorder=rec, **kw)


def _every(name):
    return TR.IntervalController(interval=C.CASES[name]["record"])


def _golden_traj(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))["traj"]


@pytest.mark.parametrize("name", RECORDED)
def test_cpu_recorder_matches_the_reference_and_the_device_recorder(name):
    cpu = _integrate(name, TR.CPURecorder(_every(name)))
    auto = _integrate(name, TR.AutoRecorder(_every(name)))
    assert cpu.device.type == "cpu" and auto.device.type == "cuda"
    assert S.rel_l2(cpu.numpy(), _golden_traj(name)) <= TOL
    assert torch.equal(cpu, auto.cpu())


@pytest.mark.parametrize("name", RECORDED)
def test_cpu_recorder_in_fourier_space(name):
    spec = _integrate(name, TR.CPURecorder(_every(name)), return_in_fourier=True)
    assert spec.is_complex() and spec.device.type == "cpu"
    nd = len(C.CASES[name]["mesh"])
    phys = torch.fft.ifftn(spec.to(torch.complex128), dim=tuple(range(-nd, 0))).real
    assert S.rel_l2(phys.numpy(), _golden_traj(name)) <= TOL


@pytest.mark.parametrize("fmt", ["torch", "numpy"])
@pytest.mark.parametrize("name", RECORDED)
def test_disk_recorder_chunks_concatenate_to_the_reference_trajectory(tmp_path, name, fmt):
    rec = TR.DiskRecorder(_every(name), cache_dir=str(tmp_path) + os.sep, cache_freq=2, save_format=fmt)
    assert _integrate(name, rec) is None
    names = sorted(os.listdir(tmp_path), key=lambda n: int(n.split("_")[-1].split(".")[0]))
    frames = _golden_traj(name).shape[1]
    assert len(names) == (frames + 1) // 2
    chunks = [torch.load(tmp_path / n) if fmt == "torch" else torch.from_numpy(np.load(tmp_path / n))
              for n in names]
    got = torch.cat(chunks, dim=1)
    assert S.rel_l2(got.numpy(), _golden_traj(name)) <= TOL


def test_random_batch_wised_recorder_frames_on_the_plane_passes():
    name = "ns2d_n32"  # 2 samples, 50 steps
    auto = _integrate(name, TR.AutoRecorder())  # every step: 51 frames
    np.random.seed(11)
    rec = TR.RandomBatchWisedRecorder(simulation_steps=50, recorder_interval=5, n_recorded_frames=3)
    out = _integrate(name, rec)
    ids = rec._recorded_frame_id
    assert out.shape == (2, 3, 1, 32, 32) and ids.shape == (2, 3)
    for b in range(2):
        assert np.all(np.diff(ids[b]) == 5)
        assert S.rel_l2(out[b].cpu().numpy(), auto[b, ids[b]].cpu().numpy()) <= 1e-6
    # the golden trajectory holds every 10th step: compare the frames that fall on it
    g = _golden_traj(name)
    for b in range(2):
        for j, step in enumerate(ids[b]):
            if step % 10 == 0:
                assert S.rel_l2(out[b, j].cpu().numpy(), g[b, step // 10]) <= TOL


def test_interval_controller_start_on_the_line_kernel():
    name = "ks1d_n128"  # 100 steps, frames every 20
    ctl = TR.IntervalController(interval=20, start=40)
    out = _integrate(name, TR.AutoRecorder(ctl))
    assert S.rel_l2(out.cpu().numpy(), _golden_traj(name)[:, 2:]) <= TOL
