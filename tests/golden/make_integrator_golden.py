"""Generate tests/golden/integrator_objects.npz: integrator objects built the reference's way
(``SETDRKIntegrator.SETDRK4.value(dt, linear_coef, nonlinear_func, **cfg)``,
``ETDRKIntegrator.ETDRK0.value(dt, linear_coef)``, ``RKIntegrator.RK4.value()``; operator/_base.py
:441-526) and stepped by hand, in float64 on the CPU.

    python tests/golden/make_integrator_golden.py <reference source tree>

``problem()`` builds the linear coefficient, the nonlinear function (a dealiased Burgers-type term
written with torch only, so both packages get the same callable) and the initial spectrum;
``SCHEMES`` lists (name, enum class name, member, config, steps). ``tests/test_integrator_objects_host.py``
runs the same objects from torchfsm_gb300.
"""

from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
N, DT, STEPS = 64, 0.02, 10
DT_RK = 2e-4  # explicit schemes: dt |L| <= 0.5 at the highest mode

SCHEMES = [
    ("etdrk0", "ETDRKIntegrator", "ETDRK0", {}),
    ("etdrk1", "ETDRKIntegrator", "ETDRK1", {}),
    ("etdrk2", "ETDRKIntegrator", "ETDRK2", {}),
    ("setdrk1", "SETDRKIntegrator", "SETDRK1", {}),
    ("setdrk2", "SETDRKIntegrator", "SETDRK2", {}),
    ("setdrk3", "SETDRKIntegrator", "SETDRK3", {}),
    ("setdrk4", "SETDRKIntegrator", "SETDRK4", {}),
    ("setdrk4_m32_r2", "SETDRKIntegrator", "SETDRK4", {"n_integration_points": 32, "integration_radius": 2.0}),
    ("rk4", "RKIntegrator", "RK4", {}),
    ("dorpi45", "RKIntegrator", "Dorpi45", {}),
    ("rk4_38rule", "RKIntegrator", "RK4_38Rule", {}),
]


def problem():
    """(linear coefficient [1, 1, N], nonlinear function of a full spectrum, u_hat0 [2, 1, N]),
    complex128 on the CPU; L = 0.05 d^2/dx^2 - 0.002 d^4/dx^4 on [0, 2 pi)."""
    import torch

    k = torch.fft.fftfreq(N, d=1.0 / N, dtype=torch.float64)
    L = (-0.05 * k ** 2 - 0.002 * k ** 4).to(torch.complex128).reshape(1, 1, N)
    keep = (k.abs() <= N / 3).to(torch.float64).reshape(1, 1, N)
    ik = (1j * k).reshape(1, 1, N)

    def nonlinear(u_hat):
        u = torch.fft.ifft(u_hat * keep).real
        return -0.5 * ik * torch.fft.fft(u * u)

    rng = np.random.Generator(np.random.PCG64(42))
    x = np.arange(N) / N * 2 * math.pi
    u0 = np.stack([np.sin(x) + 0.3 * np.cos(3 * x + rng.uniform(0, 6)), 0.5 * np.cos(2 * x)])[:, None]
    return L, nonlinear, torch.fft.fft(torch.tensor(u0))


def run(M, name, enum_name, member, cfg):
    """Final spectrum after STEPS steps of the named integrator object of namespace ``M``."""
    L, nonlinear, u = problem()
    enum = getattr(M.integrator, enum_name)
    value = getattr(enum, member).value
    if enum_name == "RKIntegrator":
        obj = value(**cfg)
        for _ in range(STEPS):
            u = obj.step(lambda x: L * x + nonlinear(x), u, DT_RK)
        return u
    obj = value(DT, L, **cfg) if member == "ETDRK0" else value(DT, L, nonlinear, **cfg)
    assert obj.dt == DT
    for _ in range(STEPS):
        u = obj.step(u)
    return u


def main(ref_root: str) -> None:
    sys.path.insert(0, ref_root)
    sys.path.insert(0, HERE)
    sys.path.insert(0, REPO)
    import cases as C

    M = C.namespace("torchfsm")
    out = {name: run(M, name, e, m, cfg).numpy() for name, e, m, cfg in SCHEMES}
    np.savez(os.path.join(HERE, "integrator_objects.npz"), **out)
    print("wrote", sorted(out))


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TORCHFSM_REFERENCE")
    if not ref:
        sys.exit(f"usage: python {os.path.relpath(__file__)} <reference source tree> (or set TORCHFSM_REFERENCE)")
    main(ref)
