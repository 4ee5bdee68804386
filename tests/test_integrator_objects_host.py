"""Integrator objects built the reference's way (``Enum.member.value(...)``), on the CPU.

``tests/golden/make_integrator_golden.py`` builds ETDRK0-2, SETDRK1-4 (and SETDRK4 with M = 32,
r = 2) integrators as ``enum.value(dt, linear_coef[, nonlinear_func], **cfg)`` and Runge-Kutta
ones as ``enum.value()``, steps them by hand ten times and stores the reference's float64 result.
The same calls on torchfsm_gb300's enums must agree: the ETD objects step through the library
(here its CPU stand-ins from ``tests/cpu_library.py``, FP32 half spectra: rel-L2 <= 1e-5), the
Runge-Kutta objects apply their tableau to the given function in its own dtype (1e-12).
"""

import os

import numpy as np
import pytest
import torch

import cases as C
import cpu_library as CL
import make_integrator_golden as G
from oracle import spectral as S
from torchfsm_gb300.integrator import RKIntegrator, SETDRKIntegrator
from torchfsm_gb300.integrator._standalone import RK_TABLES

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "integrator_objects.npz")


@pytest.mark.parametrize("name,enum_name,member,cfg", G.SCHEMES, ids=[s[0] for s in G.SCHEMES])
def test_integrator_object_matches_reference(name, enum_name, member, cfg, monkeypatch):
    CL.install(monkeypatch)
    ref = np.load(GOLDEN)[name]
    got = G.run(C.namespace("torchfsm_gb300"), name, enum_name, member, cfg).numpy()
    assert got.shape == ref.shape and np.isfinite(ref).all()
    tol = 1e-12 if enum_name == "RKIntegrator" else 1e-5
    assert np.linalg.norm(got - ref) <= tol * np.linalg.norm(ref)


def test_enum_values_are_the_library_codes():
    assert int(SETDRKIntegrator.SETDRK4.value) == 14 and SETDRKIntegrator.SETDRK4.value == 14
    assert len({m.value for m in RKIntegrator}) == 10


def test_tableaus_equal_the_oracles():
    for member in RKIntegrator:
        rows, weights = RK_TABLES[int(member.value)]
        o_rows, o_weights = S.RK_TABLEAUS[member.name]
        assert [list(map(float, r)) for r in rows] == [list(map(float, r)) for r in o_rows]
        assert list(map(float, weights)) == list(map(float, o_weights))


def test_adaptive_objects_are_not_provided():
    with pytest.raises(NotImplementedError):
        RKIntegrator.Dorpi45.value(adaptive=True)


def test_etd_object_needs_its_nonlinear_function():
    with pytest.raises(ValueError):
        SETDRKIntegrator.SETDRK4.value(0.1, torch.zeros(1, 1, 16, dtype=torch.complex128))
