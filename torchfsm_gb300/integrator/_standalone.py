"""Integrator objects built the reference's way: ``Enum.member.value(...)``.

The reference's integrator enums hold classes, and its ``_build_integrator``
(operator/_base.py:441-526) constructs them as ``SETDRKIntegrator.SETDRK4.value(dt, linear_coef,
nonlinear_func, **cfg)`` (ETDRK0: ``value(dt, linear_coef)``) or ``RKIntegrator.RK4.value(**cfg)``;
code that drives its own loop can do the same. Here the enum values are the library's scheme
codes, callable with those arguments:

* ``ETDIntegrator``: ``.dt``, ``.step(u_hat)`` and ``.forward(u_hat, dt)`` on full spectra
  [B, C, n..] of real fields. On the first step for a grid (and device) it builds a library plan
  of the linear coefficient (the FP64 coefficient kernel's tables) and steps the half spectrum
  with the library: the pointwise kernel for ETDRK0, the stage recurrences of the callback path
  around ``nonlinear_func`` (full spectrum in, full spectrum out) for the others.
* ``RKStepper``: ``.step(f, x_t, dt)`` with the scheme's Butcher tableau
  (integrator/_rk.py:43-58), for any tensor-valued ``f``; fixed step only, as in ``integrate``.
"""

from __future__ import annotations

from typing import Callable, Optional

import torch

from .. import _lib

# Butcher tableaus: rows (c_i, a_i1, a_i2, ..) and weights b, in the reference's row layout
# (integrator/_rk.py:82-255). Each stage's input sums a_ij k_j over the slopes available, the
# first entry of a row being c_i; the 3/8 rule's last row is read that way too, as the reference
# reads it.
RK_TABLES = {
    _lib.FSM_RK_EULER: ([[1.0]], [1.0]),
    _lib.FSM_RK_MIDPOINT: ([[1 / 2, 1 / 2]], [0, 1]),
    _lib.FSM_RK_HEUN12: ([[1, 1]], [1 / 2, 1 / 2]),
    _lib.FSM_RK_RALSTON12: ([[2 / 3, 2 / 3]], [1 / 4, 3 / 4]),
    _lib.FSM_RK_BOGACKI_SHAMPINE23: ([[1 / 2, 1 / 2], [3 / 4, 0, 3 / 4], [1, 2 / 9, 1 / 3, 4 / 9]],
                                     [2 / 9, 1 / 3, 4 / 9, 0]),
    _lib.FSM_RK4: ([[1 / 2, 1 / 2], [1 / 2, 0, 1 / 2], [1, 0, 0, 1]], [1 / 6, 1 / 3, 1 / 3, 1 / 6]),
    _lib.FSM_RK4_38RULE: ([[1 / 3, 1 / 3], [2 / 3, -1 / 3, 1], [1, -1, 1, 1]], [1 / 8, 3 / 8, 3 / 8, 1 / 8]),
    _lib.FSM_RK_DORPI45: ([[1 / 5, 1 / 5], [3 / 10, 3 / 40, 9 / 40], [4 / 5, 44 / 45, -56 / 15, 32 / 9],
                           [8 / 9, 19372 / 6561, -25360 / 2187, 64448 / 6561, -212 / 729],
                           [1, 9017 / 3168, -355 / 33, 46732 / 5247, 49 / 176, -5103 / 18656],
                           [1, 35 / 384, 0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84]],
                          [35 / 384, 0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84]),
    _lib.FSM_RK_FEHLBERG45: ([[1 / 4, 1 / 4], [3 / 8, 3 / 32, 9 / 32],
                              [12 / 13, 1932 / 2197, -7200 / 2197, 7296 / 2197],
                              [1, 439 / 216, -8, 3680 / 513, -845 / 4104],
                              [1 / 2, -8 / 27, 2, -3544 / 2565, 1859 / 4104, -11 / 40]],
                             [16 / 135, 0, 6656 / 12825, 28561 / 56430, -9 / 50, 2 / 55]),
    _lib.FSM_RK_CASHKARP45: ([[1 / 5, 1 / 5], [3 / 10, 3 / 40, 9 / 40], [3 / 5, 3 / 10, -9 / 10, 6 / 5],
                              [1, -11 / 54, 5 / 2, -70 / 27, 35 / 27],
                              [7 / 8, 1631 / 55296, 175 / 512, 575 / 13824, 44275 / 110592, 253 / 4096]],
                             [37 / 378, 0, 250 / 621, 125 / 594, 0, 512 / 1771]),
}

ETD_SCHEMES = (_lib.FSM_ETDRK0, _lib.FSM_ETDRK1, _lib.FSM_ETDRK2, _lib.FSM_SETDRK1, _lib.FSM_SETDRK2,
               _lib.FSM_SETDRK3, _lib.FSM_SETDRK4)


class ETDIntegrator:
    """An ETD integrator object (the reference's protocol: ``dt``, ``step(u_hat)``,
    ``forward(u_hat, dt)``) over the library, for full spectra of real fields."""

    def __init__(self, scheme: int, dt: float, linear_coef, nonlinear_func: Optional[Callable] = None,
                 n_integration_points: int = 16, integration_radius: float = 1.0, cpu_cached: bool = False):
        if scheme not in ETD_SCHEMES:
            raise ValueError(f"not an ETD scheme: {scheme}")
        if scheme != _lib.FSM_ETDRK0 and nonlinear_func is None:
            raise ValueError("this scheme needs a nonlinear function")
        self.scheme = int(scheme)
        self.dt = float(dt)
        self.linear_coef = linear_coef
        self.nonlinear_func = nonlinear_func
        self.n_integration_points = int(n_integration_points)
        self.integration_radius = float(integration_radius)
        self._plans = {}

    def _plan_for(self, u_hat: torch.Tensor):
        from .. import _native
        from ._callback import ClosurePlan

        shape = tuple(int(n) for n in u_hat.shape[2:])
        key = (shape, u_hat.shape[1], u_hat.device)
        if key not in self._plans:
            nd = len(shape)
            # the tables and transforms depend on the grid's sizes and the coefficient's values only
            mesh_info = tuple((0.0, 1.0, n) for n in shape)
            prog = _native.SpectralProgram(mesh_info, int(u_hat.shape[1]),
                                           keep=[torch.ones(n, dtype=torch.uint8) for n in shape])
            L = torch.as_tensor(self.linear_coef).to(device=u_hat.device, dtype=torch.complex128)
            if L.dim() < nd + 2:  # the reference's [0.0] when there is no linear term
                L = L.reshape((1, 1) + (1,) * nd)
            L = L.expand(tuple(L.shape[:2]) + shape)
            plan = _native.NativePlan(prog, self.dt, self.scheme, u_hat.device,
                                      n_integration_points=self.n_integration_points,
                                      integration_radius=self.integration_radius, linear_coef64=L)
            stepper = plan if self.scheme == _lib.FSM_ETDRK0 else ClosurePlan(plan, self.nonlinear_func)
            self._plans[key] = (stepper, _native.Spectral(plan))
        return self._plans[key]

    @torch.no_grad()
    def step(self, u_hat: torch.Tensor) -> torch.Tensor:
        """One step of the full spectrum ``u_hat`` [B, C, n..] (its Hermitian part: real fields)."""
        stepper, sp = self._plan_for(u_hat)
        half = sp.full_to_half(u_hat).contiguous()
        stepper.integrate_half(half, 1)
        return sp.half_to_full(half).to(u_hat.dtype)

    def forward(self, u_hat: torch.Tensor, dt: float) -> torch.Tensor:
        return self.step(u_hat)


class RKStepper:
    """An explicit Runge-Kutta integrator object (the reference's protocol: ``step(f, x_t, dt)``)."""

    def __init__(self, scheme: int, adaptive: bool = False, atol: float = 1e-6, rtol: float = 1e-5):
        if adaptive:
            raise NotImplementedError("adaptive step-size control of the Runge-Kutta integrators is not provided "
                                      "by torchfsm_gb300; the fixed-step schemes are")
        self.scheme = int(scheme)
        self.rows, self.weights = RK_TABLES[self.scheme]
        self.adaptive, self.atol, self.rtol = False, atol, rtol

    def step(self, f: Callable[[torch.Tensor], torch.Tensor], x_t: torch.Tensor, dt: float) -> torch.Tensor:
        """x_t + dt sum_i b_i k_i with k_0 = f(x_t) and k_i = f(x_t + dt sum_j a_ij k_j), each sum over
        the slopes available."""
        slopes = [f(x_t)]
        for row in self.rows:
            slopes.append(f(x_t + dt * sum(a * k for a, k in zip(row[1:], slopes))))
        return x_t + dt * sum(w * k for w, k in zip(self.weights, slopes))


class SchemeCode(int):
    """An integrator enum value: the library's scheme code, callable like the reference's enum
    values (which are classes) to build an integrator object."""

    def __new__(cls, code: int):
        return int.__new__(cls, code)

    def __call__(self, *args, **kwargs):
        if int(self) in RK_TABLES:
            return RKStepper(int(self), *args, **kwargs)
        return ETDIntegrator(int(self), *args, **kwargs)
