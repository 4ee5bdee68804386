"""Small helpers with the reference's semantics (torchfsm/utils.py)."""

from __future__ import annotations

import gc
from typing import Optional, Tuple, Union

import torch


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
