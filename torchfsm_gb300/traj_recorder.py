"""Trajectory recorders with the reference's protocol (torchfsm/traj_recorder.py).

A recorder is called as ``record(step, frame_fft)`` before every step and
after the last one (operator/_base.py:731-746) and decides with its
``control_func`` which frames to keep; ``trajectory`` returns them stacked
as [B, T, C, n1, ..] in physical space, or as spectra when
``return_in_fourier`` is set (traj_recorder.py:46-125).

The fused integrate path does not call ``record`` per step: it evaluates
``control_func`` for every step up front and lets the CUDA kernels write the
selected frames (as half spectra) straight into one device buffer, which is
handed to the recorder as a block. Frames recorded through ``record``
(custom recorders, the per-step path) are accepted as full spectra.
"""

from __future__ import annotations

import os
from typing import Callable, List, Literal, Optional

import numpy as np
import torch

from .utils import default


class IntervalController:
    """Record every ``interval`` steps from ``start`` on (traj_recorder.py:7-22)."""

    def __init__(self, interval: int = 1, start: int = 0) -> None:
        self.start = start
        self.interval = interval

    def __call__(self, step: int) -> bool:
        return step >= self.start and (step - self.start) % self.interval == 0


class _TrajRecorder:
    """Base recorder (traj_recorder.py:24-93)."""

    def __init__(self, control_func: Optional[Callable[[int], bool]] = None, include_initial_state: bool = True):
        control_func = default(control_func, lambda step: True)
        if include_initial_state:
            self.control_func = control_func
        else:
            self.control_func = lambda step: False if step == 0 else control_func(step)
        self.return_in_fourier = False

    def record(self, step: int, frame: torch.Tensor):
        if self.control_func(step):
            self._record(step, frame)

    def _record(self, step: int, frame: torch.Tensor):
        raise NotImplementedError

    def _traj_ifft(self, trajectory: torch.Tensor) -> torch.Tensor:
        fft_dim = tuple(-(i + 1) for i in range(trajectory.dim() - 3))
        return torch.fft.ifftn(trajectory, dim=fft_dim)

    @property
    def trajectory(self):
        raise NotImplementedError

    # -- fused-path protocol ------------------------------------------------
    def _accepts_blocks(self) -> bool:
        return False


class _Block:
    """Frames written by the kernels: half spectra [B, T, C, S] plus their transform."""

    def __init__(self, half: torch.Tensor, spectral):
        self.half = half
        self.spectral = spectral  # torchfsm_gb300._native.Spectral


class AutoRecorder(_TrajRecorder):
    """Keep the frames on the simulation's device (traj_recorder.py:95-125)."""

    def __init__(self, control_func: Optional[Callable[[int], bool]] = None, include_initial_state: bool = True):
        super().__init__(control_func, include_initial_state)
        self._trajectory: List = []

    def _record(self, step: int, frame: torch.Tensor):
        if isinstance(self._trajectory, torch.Tensor):
            raise RuntimeError("The trajectory has been finalized.")
        self._trajectory.append(frame.clone())

    def _accepts_blocks(self) -> bool:
        # a subclass that overrides the per-step hooks keeps the per-step protocol
        return type(self).record is _TrajRecorder.record and type(self)._record in (
            AutoRecorder._record, CPURecorder._record)

    def _add_block(self, half: torch.Tensor, spectral) -> None:
        self._trajectory.append(_Block(self._place(half), spectral))

    def _place(self, t: torch.Tensor) -> torch.Tensor:
        return t

    def _half_frames(self) -> torch.Tensor:
        """All frames as half spectra [B, T, C, S] (complex64)."""
        parts = []
        spectral = None
        for e in self._trajectory:
            if isinstance(e, _Block):
                parts.append(e.half)
                spectral = e.spectral
        if len(parts) != len(self._trajectory):
            raise RuntimeError("mixed recording modes")
        return torch.cat(parts, dim=1), spectral

    @property
    def trajectory(self):
        if len(self._trajectory) == 0:
            return None
        if all(isinstance(e, _Block) for e in self._trajectory):
            half, spectral = self._half_frames()
            if self.return_in_fourier:
                return spectral.half_to_full(half)
            return spectral.to_physical(half)
        frames = []
        for e in self._trajectory:
            if isinstance(e, _Block):
                frames.extend(e.spectral.half_to_full(e.half).unbind(1))
            else:
                frames.append(e)
        traj = torch.stack(frames, dim=1)
        if self.return_in_fourier:
            return traj
        return self._traj_ifft(traj).real


class CPURecorder(AutoRecorder):
    """Keep the frames in host memory (traj_recorder.py:127-148)."""

    def _record(self, step: int, frame: torch.Tensor):
        self._trajectory.append(frame.clone() if frame.is_cpu else frame.cpu())

    def _place(self, t: torch.Tensor) -> torch.Tensor:
        return t.cpu()

    @property
    def trajectory(self):
        if len(self._trajectory) == 0:
            return None
        if all(isinstance(e, _Block) for e in self._trajectory):
            half, spectral = self._half_frames()
            dev = spectral.device
            if self.return_in_fourier:
                return spectral.half_to_full(half.to(dev)).cpu()
            return spectral.to_physical(half.to(dev)).cpu()
        return super().trajectory


class DiskRecorder(_TrajRecorder):
    """Write frames to disk in chunks of ``cache_freq`` frames (traj_recorder.py:150-204).

    The reference's chunk test is broken (``len(self.traj<...)``); this one
    buffers ``cache_freq`` frames, then stacks them to [B, T, C, ..], converts
    them to physical space unless ``return_in_fourier`` and saves
    ``temp_cache_{step}`` (``step`` = the chunk's last recorded step) with
    torch.save or np.save (``.npy``). Reading ``trajectory`` -- ``integrate``
    does so after the last step -- saves the frames still buffered as a last,
    shorter chunk and returns None.
    """

    def __init__(self, control_func=None, include_initial_state: bool = True, cache_dir: Optional[str] = None,
                 cache_freq: int = 1, temp_cache_loc: Literal["auto", "cpu"] = "cpu",
                 save_format: Literal["numpy", "torch"] = "torch"):
        super().__init__(control_func, include_initial_state)
        self.cache_dir = default(cache_dir, "./saved_traj/")
        self.cache_freq = cache_freq
        if temp_cache_loc not in ("auto", "cpu"):
            raise ValueError("temp_cache_loc must be either 'auto' or 'cpu'.")
        if save_format not in ("numpy", "torch"):
            raise ValueError("save_format must be either 'numpy' or 'torch'.")
        self.temp_cache_loc = temp_cache_loc
        self.save_format = save_format
        self._trajectory: List[torch.Tensor] = []
        self._last_step = 0

    def _record(self, step: int, frame: torch.Tensor):
        keep = frame.cpu() if (self.temp_cache_loc == "cpu" and not frame.is_cpu) else frame.clone()
        self._trajectory.append(keep)
        self._last_step = step
        if len(self._trajectory) >= self.cache_freq:
            self._flush(step)

    def _flush(self, step: int):
        if not self._trajectory:
            return
        chunk = torch.stack(self._trajectory, dim=1)
        chunk = chunk.cpu()
        if not self.return_in_fourier:
            chunk = self._traj_ifft(chunk).real
        os.makedirs(self.cache_dir, exist_ok=True)
        path = os.path.join(self.cache_dir, f"temp_cache_{step}")
        if self.save_format == "numpy":
            np.save(path, chunk.numpy())
        else:
            torch.save(chunk, path)
        self._trajectory = []

    @property
    def trajectory(self):
        if self._trajectory:
            self._flush(self._last_step)
        return None


class RandomBatchWisedRecorder(_TrajRecorder):
    """Per sample, ``n_recorded_frames`` frames ``recorder_interval`` apart from a random
    start (traj_recorder.py:206-264)."""

    def __init__(self, simulation_steps: int, recorder_interval: int, n_recorded_frames: int = 2):
        super().__init__(None, False)
        self.simulation_steps = simulation_steps
        self.recorder_interval = recorder_interval
        self.n_recorded_frames = n_recorded_frames
        self._trajectory = []
        self._batch_size = None
        self._recorded_frame_id = None

    def _initialize_recording(self, batch_size: int):
        self._batch_size = batch_size
        first = np.random.randint(1, self.simulation_steps - self.recorder_interval * self.n_recorded_frames,
                                  size=batch_size)
        self._recorded_frame_id = np.stack([first + i * self.recorder_interval for i in range(self.n_recorded_frames)], 1)
        self._trajectory = [[] for _ in range(batch_size)]

    def record(self, step: int, frame: torch.Tensor):
        if self._batch_size is None:
            self._initialize_recording(frame.shape[0])
        for b in range(self._batch_size):
            if step in self._recorded_frame_id[b]:
                self._trajectory[b].append(frame[b].clone())

    @property
    def trajectory(self):
        if len(self._trajectory) == 0:
            return None
        trajs = torch.stack([torch.stack(t, dim=0) for t in self._trajectory], dim=0)
        self._trajectory = []
        if self.return_in_fourier:
            return trajs
        return self._traj_ifft(trajs).real
