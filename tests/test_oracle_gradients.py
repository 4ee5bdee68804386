"""The reference's autograd gradients (golden) against central finite differences of the FP64 oracle."""

import os

import numpy as np
import pytest

import cases as C
from oracle import spectral as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _loss(name, u0, nu):
    c = C.GRAD_CASES[name]
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    out, _ = S.integrate(u0, c["mesh"], [(nu, ("laplacian",))], [(-1.0, "convection")], c["dt"], c["step"])
    return float(np.mean((out - g["target"]) ** 2))


@pytest.mark.parametrize("name", sorted(C.GRAD_CASES))
def test_reference_gradients_match_central_differences(name):
    c = C.GRAD_CASES[name]
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    u0 = g["u0"]
    assert abs(_loss(name, u0, c["nu"]) - float(g["loss"])) <= 1e-10 * float(g["loss"])
    eps = 1e-3
    fd_nu = (_loss(name, u0, c["nu"] + eps) - _loss(name, u0, c["nu"] - eps)) / (2 * eps)
    assert abs(fd_nu - float(g["grad_nu"])) <= 1e-3 * abs(float(g["grad_nu"]))
    v = np.random.default_rng(0).standard_normal(u0.shape)
    v /= np.linalg.norm(v)
    fd_u = (_loss(name, u0 + eps * v, c["nu"]) - _loss(name, u0 - eps * v, c["nu"])) / (2 * eps)
    ad_u = float(np.sum(g["grad_u0"] * v))
    assert abs(fd_u - ad_u) <= 1e-3 * abs(ad_u) + 1e-12


_GENERIC_TERMS = {
    "grad_ns2d_n32": lambda c: ([(c, ("laplacian",))], [(-1.0, "vorticity_convection")]),
    "grad_ksnd2d_n32": lambda c: ([(c, ("laplacian",)), (-1.0, ("biharmonic",))], [(-1.0, "ks_convection")]),
    "grad_kdv1d_n64": lambda c: ([(c, ("spatial_derivative", 0, 3))], [(6.0, "convection")]),
    "grad_burgers1d_etdrk2_n64": lambda c: ([(c, ("laplacian",))], [(-1.0, "convection")]),
    "grad_burgers2d_setdrk3_n32": lambda c: ([(c, ("laplacian",))], [(-1.0, "convection")]),
    "grad_burgers1d_rk4_n64": lambda c: ([(c, ("laplacian",))], [(-1.0, "convection")]),
    "grad_heat2d_etdrk0_n16": lambda c: ([(c, ("laplacian",))], []),
}


def _generic_loss(name, u0, coef):
    c = C.GENERIC_GRAD_CASES[name]
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    lin, nl = _GENERIC_TERMS[name](coef)
    integ = c.get("integrator", "auto")
    out, _ = S.integrate(u0, c["mesh"], lin, nl, c["dt"], c["step"], integrator=integ if integ in S.RK_TABLEAUS
                         else integ.lower())
    return float(np.mean((out - g["target"]) ** 2))


@pytest.mark.parametrize("name", sorted(C.GENERIC_GRAD_CASES))
def test_reference_gradients_of_other_programs_match_central_differences(name):
    c = C.GENERIC_GRAD_CASES[name]
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    u0 = g["u0"]
    assert abs(_generic_loss(name, u0, c["coef"]) - float(g["loss"])) <= 1e-9 * float(g["loss"])
    eps = 1e-4
    fd_c = (_generic_loss(name, u0, c["coef"] + eps) - _generic_loss(name, u0, c["coef"] - eps)) / (2 * eps)
    assert abs(fd_c - float(g["grad_coef"])) <= 1e-3 * abs(float(g["grad_coef"]))
    v = np.random.default_rng(1).standard_normal(u0.shape)
    v /= np.linalg.norm(v)
    fd_u = (_generic_loss(name, u0 + eps * v, c["coef"]) - _generic_loss(name, u0 - eps * v, c["coef"])) / (2 * eps)
    ad_u = float(np.sum(g["grad_u0"] * v))
    assert abs(fd_u - ad_u) <= 1e-3 * abs(ad_u) + 1e-12
