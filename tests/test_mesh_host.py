"""The mesh classes against the reference's (CPU, float64).

Each query of ``tests/golden/make_mesh_golden.py`` -- coordinates (whose start offsets the
reference ignores), broadcast grids, FFT frequencies, their broadcast forms, the derivative and
Laplacian symbols and their inverses, the dealias and absolute low-pass masks, ``mesh_shape`` --
runs on ``torchfsm_gb300.mesh`` and must equal the reference's answer (golden vectors made by
the reference itself) in shape, dtype and, to 1e-12, value. These symbols are what the library's
FP64 coefficient kernel and the dealias masks of the fused kernels are built from.
"""

import os

import numpy as np
import pytest

import make_mesh_golden as G
from torchfsm_gb300 import mesh

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mesh_reference.npz")


@pytest.mark.parametrize("name,query", G.QUERIES, ids=[q[0] for q in G.QUERIES])
def test_mesh_query_matches_reference(name, query):
    ref = np.load(GOLDEN)[name]
    got = query(mesh)
    got = np.asarray(got) if isinstance(got, tuple) else got.numpy()
    assert got.shape == ref.shape, (got.shape, ref.shape)
    assert got.dtype == ref.dtype, (got.dtype, ref.dtype)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)
