"""Generate tests/golden/field_helpers.npz by running the reference's initial-condition helpers
(torchfsm/field.py) under fixed torch seeds.

    python tests/golden/make_field_golden.py <reference source tree>

``CALLS`` lists each helper call: a name, the torch seed set before it, and a function that
makes the call on a given ``field`` module (the reference's when generating, torchfsm_gb300's in
``tests/test_field_host.py``). The reference is imported from the given source tree (CPU only).
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _x(n: int, batch: int = 0):
    import torch

    x = (torch.arange(n, dtype=torch.float64) / n).reshape(1, n)
    return x.reshape(1, 1, n).repeat(batch, 1, 1) if batch else x


CALLS = [
    ("tfs_1d", 0, lambda F: F.truncated_fourier_series([(0, 1, 64)], freq_threshold=5, batch_size=2,
                                                       dtype=_dtype64())),
    ("tfs_2d_var", 1, lambda F: F.truncated_fourier_series([(0, 1, 32), (0, 1, 32)], freq_threshold=4,
                                                           unit_variance=True, unit_magnitude=False, batch_size=2,
                                                           n_channel=2, dtype=_dtype64())),
    ("tfs_1d_ranges", 2, lambda F: F.truncated_fourier_series([(0, 2, 48)], freq_threshold=3,
                                                              amplitude_range=(0.5, 2.0), angle_range=(0.0, 1.0),
                                                              zero_centered=False, batch_size=3,
                                                              dtype=_dtype64())),
    ("wave_1d", 3, lambda F: F.wave_1d(_x(128))),
    ("wave_1d_batched", 4, lambda F: F.wave_1d(_x(96, batch=3), min_k=2, max_k=6, n_polynomial=3, batched=True)),
    ("wave_1d_zero_mean", 5, lambda F: F.wave_1d(_x(64), zero_mean=True)),
    ("diffused_1d", 6, lambda F: F.diffused_noise([(0, 1, 64)], diffusion_coef=1e-3, batch_size=2,
                                                  dtype=_dtype64())),
    ("diffused_2d_var", 7, lambda F: F.diffused_noise([(0, 1, 32), (0, 1, 32)], diffusion_coef=5e-3,
                                                      unit_variance=True, unit_magnitude=False, n_channel=2,
                                                      dtype=_dtype64())),
]


def _dtype64():
    import torch

    return torch.float64


def main(ref_root: str) -> None:
    sys.path.insert(0, ref_root)
    import torch
    from torchfsm import field as F

    out = {}
    for name, seed, call in CALLS:
        torch.manual_seed(seed)
        out[name] = call(F).numpy()
    np.savez(os.path.join(HERE, "field_helpers.npz"), **out)
    print("wrote", os.path.join(HERE, "field_helpers.npz"), sorted(out))


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TORCHFSM_REFERENCE")
    if not ref:
        sys.exit(f"usage: python {os.path.relpath(__file__)} <reference source tree> (or set TORCHFSM_REFERENCE)")
    main(ref)
