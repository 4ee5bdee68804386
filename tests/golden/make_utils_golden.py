"""Generate tests/golden/utils_helpers.npz by running the reference's trajectory helpers
(torchfsm/utils.py:44-183) on a small seeded trajectory.

    python tests/golden/make_utils_golden.py <reference source tree>

For each helper and torch seed the file holds the reference's output; the statistics are
stored per channel. The reference is imported from the given source tree (CPU only).
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

CALLS = [("random_clip_traj", 5), ("random_select_frames", 7), ("uniformly_select_frames", 6)]
SEEDS = [3, 11]


def trajectory() -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(2024))
    return rng.standard_normal((3, 20, 2, 4, 4)).astype(np.float32)


def main(ref_root: str) -> None:
    sys.path.insert(0, ref_root)
    import torch
    from torchfsm import utils as U

    x = trajectory()
    out = {"traj": x}
    for name, arg in CALLS:
        for seed in SEEDS:
            torch.manual_seed(seed)
            out[f"{name}_{seed}"] = getattr(U, name)(torch.from_numpy(x), arg).numpy()
    means, stds, mins, maxs = U.statistics_traj([torch.from_numpy(x), torch.from_numpy(x[:2, 5:])])
    out.update(stats_mean=np.array(means), stats_std=np.array(stds), stats_min=np.array(mins),
               stats_max=np.array(maxs))
    np.savez(os.path.join(HERE, "utils_helpers.npz"), **out)
    print("wrote", os.path.join(HERE, "utils_helpers.npz"))


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TORCHFSM_REFERENCE")
    if not ref:
        sys.exit(f"usage: python {os.path.relpath(__file__)} <reference source tree> (or set TORCHFSM_REFERENCE)")
    main(ref)
