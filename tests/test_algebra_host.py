"""The operator algebra against the reference's (CPU, float64).

Each expression of ``tests/golden/make_algebra_golden.py`` -- sums, differences, negation,
scaling and division by numbers and 0-d tensors, ``op + tensor`` and ``tensor + op`` explicit
sources, the unit ImplicitSource, 2D derivative sums, vorticity / conservative / Leray-projected
convection, and the misuses the reference rejects (``2 - op``, ``op + 1.0``) -- is built with
torchfsm_gb300 and applied once with the cores' torch arithmetic in float64 (the fused FSM_APPLY
evaluation needs a GPU and is switched off here); the value must equal the reference's to
1e-10, or the same exception type must be raised.
"""

import os

import numpy as np
import pytest

import cases as C
import make_algebra_golden as G
from oracle import spectral as S
from torchfsm_gb300.operator import _base as B

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "algebra_reference.npz")


@pytest.mark.parametrize("name,mesh,channels,build", G.EXPRESSIONS, ids=[e[0] for e in G.EXPRESSIONS])
def test_expression_matches_reference(name, mesh, channels, build, monkeypatch):
    monkeypatch.setattr(B.OperatorLike, "_apply_fused", lambda self, u, u_fft: None)
    ref = np.load(GOLDEN)[name]
    got = G.evaluate(C.namespace("torchfsm_gb300"), name, mesh, channels, build)
    if ref.dtype.kind == "U":
        assert got == str(ref)
    else:
        assert not isinstance(got, str), got
        assert got.shape == ref.shape
        assert S.rel_l2(got, ref) <= 1e-10
