"""Generate tests/golden/mesh_reference.npz by querying the reference's mesh classes
(torchfsm/mesh.py: MeshGrid, FFTFrequency, BroadcastedFFTFrequency, FourierMesh, mesh_shape).

    python tests/golden/make_mesh_golden.py <reference source tree>

``QUERIES`` lists each query: a name and a function of the mesh module that returns a tensor or
a tuple of ints; ``tests/test_mesh_host.py`` runs the same queries on torchfsm_gb300.mesh. The
reference is imported from the given source tree (CPU only).
"""

from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# 1D / 2D / 3D meshes with non-zero starts (the coordinates ignore them), odd and even sizes
M1 = [(1.0, 3.0, 12)]
M2 = [(0.5, 2 * math.pi + 0.5, 8), (0.0, 4.0, 9)]
M3 = [(0.0, 2 * math.pi, 6), (-1.0, 1.0, 8), (0.0, 3.0, 5)]


def _f64():
    import torch

    return torch.float64


QUERIES = [
    ("grid1_x", lambda m: m.MeshGrid(M1, dtype=_f64()).x),
    ("grid2_item1", lambda m: m.MeshGrid(M2, dtype=_f64())[1]),
    ("grid2_mesh_grid0", lambda m: m.MeshGrid(M2, dtype=_f64()).mesh_grid()[0]),
    ("grid3_mesh_grid2", lambda m: m.MeshGrid(M3, dtype=_f64()).mesh_grid()[2]),
    ("grid2_bc1", lambda m: m.MeshGrid(M2, dtype=_f64()).bc_mesh_grid(batch_size=2, n_channels=3)[1]),
    ("grid1_bc", lambda m: m.MeshGrid(M1, dtype=_f64()).bc_mesh_grid(batch_size=2)),
    ("freq2_f1", lambda m: m.FFTFrequency(M2, dtype=_f64())[1]),
    ("freq3_f_z", lambda m: m.FFTFrequency(M3, dtype=_f64()).f_z),
    ("bfreq3_bf1", lambda m: m.BroadcastedFFTFrequency(m.FFTFrequency(M3, dtype=_f64()))[1]),
    ("bfreq2_vector", lambda m: m.BroadcastedFFTFrequency(m.FFTFrequency(M2, dtype=_f64())).bf_vector),
    ("fm2_grad_0_1", lambda m: m.FourierMesh(M2, dtype=_f64()).grad(0, 1)),
    ("fm3_grad_2_3", lambda m: m.FourierMesh(M3, dtype=_f64()).grad(2, 3)),
    ("fm3_laplacian", lambda m: m.FourierMesh(M3, dtype=_f64()).laplacian()),
    ("fm2_invert_laplacian", lambda m: m.FourierMesh(M2, dtype=_f64()).invert_laplacian()),
    ("fm2_nabla_2", lambda m: m.FourierMesh(M2, dtype=_f64()).nabla(2)),
    ("fm3_invert_nabla_1", lambda m: m.FourierMesh(M3, dtype=_f64()).invert_nabla(1)),
    ("fm3_nabla_vector_1", lambda m: m.FourierMesh(M3, dtype=_f64()).nabla_vector(1)),
    ("fm2_low_pass", lambda m: m.FourierMesh(M2, dtype=_f64()).low_pass_filter(2 / 3)),
    ("fm3_low_pass_half", lambda m: m.FourierMesh(M3, dtype=_f64()).low_pass_filter(0.5)),
    ("fm2_abs_low_pass", lambda m: m.FourierMesh(M2, dtype=_f64()).abs_low_pass_filter(1)),
    ("fm1_bf_x", lambda m: m.FourierMesh(M1, dtype=_f64()).bf_x),
    ("fm3_bf_vector", lambda m: m.FourierMesh(M3, dtype=_f64()).bf_vector),
    ("shape3", lambda m: m.mesh_shape(M3, batch_size=4, n_channel=2)),
    ("shape_fm2", lambda m: m.mesh_shape(m.FourierMesh(M2), batch_size=1, n_channel=3)),
]


def main(ref_root: str) -> None:
    sys.path.insert(0, ref_root)
    from torchfsm import mesh as R

    out = {}
    for name, query in QUERIES:
        v = query(R)
        out[name] = np.asarray(v) if isinstance(v, tuple) else v.numpy()
    np.savez(os.path.join(HERE, "mesh_reference.npz"), **out)
    print("wrote", os.path.join(HERE, "mesh_reference.npz"), len(out), "queries")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TORCHFSM_REFERENCE")
    if not ref:
        sys.exit(f"usage: python {os.path.relpath(__file__)} <reference source tree> (or set TORCHFSM_REFERENCE)")
    main(ref)
