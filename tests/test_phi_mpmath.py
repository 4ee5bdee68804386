"""The phi-functions of the SETDRK coefficient tables against 60-digit mpmath values (CPU).

The reference builds its SETDRK coefficients as means over M points of a circle of radius r
around each z = dt L (Kassam-Trefethen, integrator/_stable_etdrk/_uncached.py:8-43, 180-211),
because the closed forms lose digits to cancellation near z = 0. The library's FP64 coefficient
kernel (k_phi_tables) evaluates the same functions directly -- a 24-term Taylor series for
|z| < 0.5, the closed forms elsewhere -- whenever r^M / M! (the size of the contour mean's
deviation from the function) is below 1e-10, and takes the contour mean otherwise. These tests
pin the mathematics of both branches to high-precision values:

* the contour mean (the oracle's restatement, M = 16, r = 1) equals the functions to 1e-12;
* the kernel's series coefficients give the functions to 1e-14 for |z| < 0.5;
* the closed forms in FP64 fail near 0 (why neither is optional);
* the deviation bound picks the direct branch for the reference's default (16, 1).
"""

import math

import numpy as np
import pytest

from oracle import spectral as S

mpmath = pytest.importorskip("mpmath")
mpmath.mp.dps = 60

# z values: tiny, small, moderate, stiff (negative real, as for diffusion), oscillatory (imaginary)
ZS = [1e-9, -3e-7, 2e-5 + 1e-5j, -1e-3, 0.01j, -0.2, 0.3 - 0.2j, 0.49, -0.75, 1.3j, -2.5, -8.0, -40.0, 3.0,
      -15.0 + 4.0j]


def _phi_exact(z):
    """(s_e1, s_e2, s_h, s_a, s_b, s_c) at z in 60-digit arithmetic."""
    z = mpmath.mpc(z)
    ez = mpmath.exp(z)
    return (
        (ez - 1) / z,
        (ez - 1 - z) / z ** 2,
        (mpmath.exp(z / 2) - 1) / z,
        (-4 - z + ez * (4 - 3 * z + z ** 2)) / z ** 3,
        (2 + z + ez * (z - 2)) / z ** 3,
        (-4 - 3 * z - z ** 2 + ez * (4 - z)) / z ** 3,
    )


def _series(z, terms=24):
    """The kernel's Taylor branch: sum_k c_k z^k with, for k = 0..terms-1,
    s_e1: 1/(k+1)!, s_e2: 1/(k+2)!, s_h: 2^-(k+1)/(k+1)!, s_a: (k+1)^2/(k+3)!, s_b: (k+1)/(k+3)!,
    s_c: (1-k)/(k+3)!."""
    out = [0j] * 6
    zk = 1.0 + 0j
    for k in range(terms):
        f1, f2, f3 = math.factorial(k + 1), math.factorial(k + 2), math.factorial(k + 3)
        coefs = (1 / f1, 1 / f2, 2.0 ** -(k + 1) / f1, (k + 1) ** 2 / f3, (k + 1) / f3, (1 - k) / f3)
        out = [o + c * zk for o, c in zip(out, coefs)]
        zk *= z
    return out


def _rel(a, b):
    return abs(complex(a) - complex(b)) / max(abs(complex(b)), 1e-300)


@pytest.mark.parametrize("z", ZS)
def test_contour_mean_equals_the_functions(z):
    dt = 1.0
    lin = np.array([z], dtype=np.complex128)
    t = S.setdrk_coefs(4, lin, dt, 16, 1.0)
    exact = _phi_exact(z)
    # the reference keeps the real part of the contour means (.real, _uncached.py:191-211)
    assert _rel(t["c1"][0], mpmath.re(exact[2])) < 1e-12
    assert _rel(t["c4"][0], mpmath.re(exact[3])) < 1e-12
    assert _rel(t["c5"][0], mpmath.re(exact[4])) < 1e-12
    assert _rel(t["c6"][0], mpmath.re(exact[5])) < 1e-12
    t2 = S.setdrk_coefs(2, lin, dt, 16, 1.0)
    assert _rel(t2["c1"][0], mpmath.re(exact[0])) < 1e-12
    assert _rel(t2["c2"][0], mpmath.re(exact[1])) < 1e-12


@pytest.mark.parametrize("z", [z for z in ZS if abs(z) < 0.5])
def test_kernel_series_branch(z):
    for got, want in zip(_series(complex(z)), _phi_exact(z)):
        assert _rel(got, want) < 1e-14


def test_closed_forms_cancel_near_zero():
    z = 1e-6
    naive = (np.exp(z) - 1 - z) / z ** 2  # s_e2 in FP64
    assert _rel(naive, _phi_exact(z)[1]) > 1e-6
    assert _rel(_series(z)[1], _phi_exact(z)[1]) < 1e-15


@pytest.mark.parametrize("m,r,direct", [(16, 1.0, True), (32, 2.0, True), (6, 1.5, False), (8, 4.0, False)])
def test_direct_branch_bound(m, r, direct):
    # r^M / M!, the size of the contour mean's deviation from the function (the M-th Taylor term)
    bound = math.exp(m * math.log(r) - math.lgamma(m + 1))
    assert (bound < 1e-10) == direct
    if direct:
        # where the bound is small, the contour mean and the function agree to it
        for z in (0.3, -2.0, 1.5j):
            t = S.setdrk_coefs(4, np.array([z], dtype=np.complex128), 1.0, m, r)
            assert _rel(t["c4"][0], mpmath.re(_phi_exact(z)[3])) < max(1e-12, 10 * bound)
