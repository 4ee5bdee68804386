"""Time stepping of programs whose nonlinear terms have no fused kernel.

A Python-callable source (``ImplicitSource(f)``), a user ``NonlinearFunc`` core,
``ConservativeConvection``, several kinds of nonlinear term in one program, or a
tensor coefficient on a nonlinear term cannot be compiled into the CUDA kernels.
Such programs step here, on the device that holds the state:

* the linear part's coefficient tables come from a library plan of the linear
  part alone (the FP64 coefficient kernel, rounded to FP32: the tables the fused
  kernels read for the same operator, mesh and dt);
* the state is the half spectrum of the fused path, and the dealiased physical
  field each nonlinear evaluation needs comes from the library's inverse
  transform;
* the operator's cores are called on full spectra with the reference's
  arguments ``(u_fft, f_mesh, u)`` and summed with their coefficients as in the
  reference's nonlinear closure (operator/_base.py:375-403);
* the stage recurrences are the reference's (ETDRK1/2: integrator/_etdrk.py:30-82;
  SETDRK1-4: integrator/_stable_etdrk/_setdrk_step.py:5-82), in torch arithmetic
  on the half spectra.

There is no CPU path: the plan, the state and the cores' arithmetic live on one
CUDA device. The explicit Runge-Kutta schemes are not offered for these
programs (``UnsupportedProgram``).
"""

from __future__ import annotations

import math
from typing import Callable, Optional, Sequence, Tuple

import torch

from .. import _lib

# schemes whose stage recurrences this module runs
CALLBACK_SCHEMES = (_lib.FSM_ETDRK1, _lib.FSM_ETDRK2, _lib.FSM_SETDRK1, _lib.FSM_SETDRK2,
                    _lib.FSM_SETDRK3, _lib.FSM_SETDRK4)

# coefficient tables per scheme, in the library's order (fsm_plan_tables)
_NTAB = {_lib.FSM_ETDRK1: 2, _lib.FSM_ETDRK2: 3, _lib.FSM_SETDRK1: 2, _lib.FSM_SETDRK2: 3,
         _lib.FSM_SETDRK3: 7, _lib.FSM_SETDRK4: 6}


class CallbackPlan:
    """A library plan of the linear part plus the operator's nonlinear cores as Python callables.

    It has the plan interface ``integrate`` uses (``integrate_half``, ``device``, ``dt``,
    ``shape``, ``handle`` for the transforms), so the operator's integrator, recorders and
    trajectory handling stay the ones of the fused path.

    ``linear_plan``: a plan of the linear part alone (no nonlinear term, no source) for the
    scheme ``linear_plan.integrator``; ``nonlinear_terms``: the operator's ``(coef, core)``
    pairs; ``f_mesh``: its registered FourierMesh; ``de_aliasing_rate``: the 2/3 rule's rate.
    """

    def __init__(self, linear_plan, nonlinear_terms: Sequence[Tuple[object, Callable]], f_mesh,
                 de_aliasing_rate: float):
        from .. import _native

        scheme = int(linear_plan.integrator)
        if scheme not in CALLBACK_SCHEMES:
            raise _lib.UnsupportedProgram(_lib.FSM_ERR_UNSUPPORTED,
                                          "terms without a fused kernel step with ETDRK1/2 or SETDRK1-4 only")
        self.inner = linear_plan
        self.integrator = scheme
        self.program = linear_plan.program
        self.dt = linear_plan.dt
        self.device = linear_plan.device
        self.shape = tuple(linear_plan.shape)
        self.n_channel = linear_plan.n_channel
        self.spectral = _native.Spectral(linear_plan)
        self.terms = list(nonlinear_terms)
        self.f_mesh = f_mesh
        h = self.shape[-1] // 2 + 1
        self.half_shape = self.shape[:-1] + (h,)
        S = math.prod(self.half_shape)
        tabs = linear_plan.tables()  # [ntab, lin_batch * lin_channel * S], the library's layout
        ntab, entries = tabs.shape
        if ntab != _NTAB[scheme] or entries % S:
            raise _lib.FsmError(_lib.FSM_ERR_INVALID, f"coefficient tables {tuple(tabs.shape)} for scheme {scheme}")
        lin_batch = max(1, int(getattr(linear_plan, "lin_batch", 1)))
        self.tables = tabs.reshape((ntab, lin_batch, entries // (S * lin_batch)) + self.half_shape)
        self.keep_half = None
        if f_mesh is not None:
            keep = f_mesh.low_pass_filter(de_aliasing_rate)
            self.keep_half = keep[..., :h].to(device=self.device, dtype=torch.float32)

    @property
    def handle(self):
        return self.inner.handle

    # -- the nonlinear closure ------------------------------------------------
    def nonlinear(self, half: torch.Tensor) -> torch.Tensor:
        """Half spectrum of sum coef * core(u) for the state's half spectrum ``half``
        (operator/_base.py:375-403): dealiasing cores get the masked spectrum and its physical
        field, the others the unmasked ones; the sum is not masked."""
        sp = self.spectral
        result = None
        d_full = d_u = full = u = None
        for coef, core in self.terms:
            if getattr(core, "_dealiasing_swtich", True):
                if d_full is None:
                    d_half = half * self.keep_half
                    d_u = sp.to_physical(d_half)
                    d_full = sp.half_to_full(d_half)
                term = core(d_full, self.f_mesh, d_u)
            else:
                if full is None:
                    u = sp.to_physical(half)
                    full = sp.half_to_full(half)
                term = core(full, self.f_mesh, u)
            if isinstance(coef, torch.Tensor):
                coef = coef.to(term.device)  # a per-sample coefficient may live on the host
            term = coef * term
            result = term if result is None else result + term
        out = sp.full_to_half(result)
        return out.to(torch.complex64)

    # -- one step ---------------------------------------------------------------
    def step(self, u: torch.Tensor) -> torch.Tensor:
        """One step of the scheme on the half spectra ``u`` [B, C, ...] (complex64).

        The library's exponential tables hold exp(dt L) - 1 (and exp(dt L / 2) - 1), so
        exp(dt L) u is formed as u + (E - 1) u, as the kernels form it."""
        T, N, s = self.tables, self.nonlinear, self.integrator

        def ex(em1, v):
            return v + em1 * v

        if s in (_lib.FSM_ETDRK1, _lib.FSM_SETDRK1):
            return ex(T[0], u) + T[1] * N(u)
        if s in (_lib.FSM_ETDRK2, _lib.FSM_SETDRK2):
            n0 = N(u)
            a1 = ex(T[0], u) + T[1] * n0
            return a1 + T[2] * (N(a1) - n0)
        if s == _lib.FSM_SETDRK3:
            n0 = N(u)
            a1 = ex(T[1], u) + T[2] * n0
            n1 = N(a1)
            Eu = ex(T[0], u)
            a2 = Eu + T[3] * (2 * n1 - n0)
            n2 = N(a2)
            return Eu + T[4] * n0 + T[5] * n1 + T[6] * n2
        n0 = N(u)  # SETDRK4
        a1 = ex(T[1], u) + T[2] * n0
        n1 = N(a1)
        a2 = ex(T[1], u) + T[2] * n1
        n2 = N(a2)
        a3 = ex(T[1], a1) + T[2] * (2 * n2 - n0)
        n3 = N(a3)
        return ex(T[0], u) + T[3] * n0 + T[4] * 2 * (n1 + n2) + T[5] * n3

    @torch.no_grad()
    def integrate_half(self, state: torch.Tensor, steps: int, slots: Optional[Sequence[int]] = None,
                       traj: Optional[torch.Tensor] = None, workspace: Optional[torch.Tensor] = None) -> None:
        """Advance half spectra [B, C, ...] (complex64) in place by ``steps`` steps; with ``slots``
        (one entry per state before each step and after the last; -1 = not recorded) the
        recorded states are written to ``traj`` [B, frames, C, ...]. ``workspace`` is not used."""
        if state.device != self.device:
            raise _lib.FsmError(_lib.FSM_ERR_INVALID, "the state is not on the plan's device")
        u = state
        for i in range(int(steps)):
            if slots is not None and slots[i] >= 0:
                traj[:, slots[i]] = u
            u = self.step(u)
        if slots is not None and slots[int(steps)] >= 0:
            traj[:, slots[int(steps)]] = u
        if u is not state:
            state.copy_(u)

    def launch_count(self, steps: int, batch: int = 0) -> int:
        """Launches of the library's own kernels (the transforms of each nonlinear evaluation;
        the cores' torch kernels are not counted)."""
        dealiased = any(getattr(c, "_dealiasing_swtich", True) for _, c in self.terms)
        plain = any(not getattr(c, "_dealiasing_swtich", True) for _, c in self.terms)
        per_eval = int(dealiased) + int(plain)
        stages = {_lib.FSM_ETDRK1: 1, _lib.FSM_SETDRK1: 1, _lib.FSM_ETDRK2: 2, _lib.FSM_SETDRK2: 2,
                  _lib.FSM_SETDRK3: 3, _lib.FSM_SETDRK4: 4}[self.integrator]
        return int(steps) * stages * int(per_eval)


class ClosurePlan(CallbackPlan):
    """The callback path around one closure on full spectra: ``closure(u_hat)`` is the whole
    nonlinear term (its dealiasing included), as an integrator constructed from the reference's
    enum protocol receives it (``SETDRKIntegrator.SETDRK4.value(dt, linear_coef, nonlinear_func)``)."""

    def __init__(self, linear_plan, closure: Callable[[torch.Tensor], torch.Tensor]):
        super().__init__(linear_plan, [], None, 1.0)
        self.closure = closure

    def nonlinear(self, half: torch.Tensor) -> torch.Tensor:
        sp = self.spectral
        return sp.full_to_half(self.closure(sp.half_to_full(half))).to(torch.complex64)

    def launch_count(self, steps: int, batch: int = 0) -> int:
        return 0

