"""Small helpers with the reference's semantics (torchfsm/utils.py)."""

from __future__ import annotations

import gc
from typing import Optional, Tuple, Union

import numpy as np
import torch

from ._type import FourierArray, FourierTensor, SpatialArray, SpatialTensor, ValueList  # noqa: F401


def default(value, default_value):
    """``value`` unless it is None (utils.py:7-18)."""
    return value if value is not None else default_value


def format_device_dtype(
    device: Optional[Union[torch.device, str]] = None,
    dtype: Optional[torch.dtype] = None,
) -> Tuple[torch.device, torch.dtype]:
    """Device defaults to CPU, "cuda" means "cuda:0", dtype defaults to float32 (utils.py:20-41)."""
    if device is None:
        device = torch.device("cpu")
    elif isinstance(device, str):
        device = torch.device(device)
    if isinstance(device, torch.device) and device.index is None and device.type != "cpu":
        device = torch.device(device.type, 0)
    return device, default(dtype, torch.float32)


def clean_up_memory() -> None:
    """Garbage-collect and release cached device memory (utils.py:185-190).

    The integrate path does not call this per step or per call: the
    reference's per-call collection costs ~0.3 s and frees nothing the fused
    path holds.
    """
    gc.collect()
    if torch.cuda.is_available():
        torch.cuda.empty_cache()


# ---- trajectory helpers for dataset building (utils.py:44-183, 192-195) -----------------------
# They act on recorded trajectories [B, T, C, ...] (tensors or numpy arrays). As in the
# reference, numpy inputs are converted to tensors and the result stays a tensor, and the random
# choices draw from torch's global generator with the same calls, so a seeded caller gets the
# same frames.


def _as_tensor(traj):
    return torch.from_numpy(traj) if isinstance(traj, np.ndarray) else traj


def statistics_traj(traj):
    """Per-channel (means, stds, mins, maxs) over batch, time and space of one trajectory or a
    list of them (utils.py:44-69); std is the unbiased estimate."""
    trajs = traj if isinstance(traj, list) else [traj]
    trajs = [_as_tensor(t) for t in trajs]
    C = trajs[0].shape[2]
    # [B, T, C, ...] -> [C, everything else]
    flat = torch.cat([t.movedim(2, 0).reshape(C, -1) for t in trajs], dim=1)
    means = [flat[c].mean().item() for c in range(C)]
    stds = [flat[c].std().item() for c in range(C)]
    mins = [flat[c].min().item() for c in range(C)]
    maxs = [flat[c].max().item() for c in range(C)]
    return means, stds, mins, maxs


def random_clip_traj(traj, length: int):
    """A random window of ``length`` frames per batch entry (utils.py:72-111): window starts are
    drawn uniformly from [0, T - length) with one torch.randint call."""
    t = _as_tensor(traj)
    starts = torch.randint(0, t.shape[1] - length, (t.shape[0],))
    return torch.stack([t[b, int(s): int(s) + length] for b, s in enumerate(starts)], dim=0)


def random_select_frames(traj, n_frames: int):
    """``n_frames`` frame indices drawn uniformly (with repetition) from [0, T), the same for every
    batch entry (utils.py:113-147)."""
    t = _as_tensor(traj)
    return t[:, torch.randint(0, t.shape[1], (n_frames,))]


def uniformly_select_frames(traj, n_frames: int):
    """``n_frames`` evenly spaced frames from the first to the last (indices truncated from
    linspace(0, T - 1, n_frames); utils.py:149-183)."""
    t = _as_tensor(traj)
    return t[:, torch.linspace(0, t.shape[1] - 1, n_frames).long()]


def print_gpu_memory(prefix: str = "", device="cuda:1") -> None:
    """Print the allocated and reserved device memory in MB (utils.py:192-195)."""
    alloc = torch.cuda.memory_allocated(device) / 1024 ** 2
    res = torch.cuda.memory_reserved(device) / 1024 ** 2
    print(f"{prefix}Allocated: {alloc:.2f} MB, Reserved: {res:.2f} MB")
