"""CPU stand-ins for the two library pieces the callback path uses (test infrastructure).

``install(monkeypatch)`` replaces, for one test:

* ``_native.NativePlan`` by a plan of a linear part whose coefficient tables are the oracle's
  FP64 tables of the same linear symbol, laid out as the library lays them out
  (``fsm_plan_tables``: [tables][lin_batch][lin_channel][half spectrum], per scheme E - 1,
  E2 - 1, c1.. in the library's order), and which steps linear ETDRK0 programs as the pointwise
  kernel does (every point plus (E - 1) times itself per step);
* ``_native.Spectral``'s forward and inverse transforms by torch's real FFTs;
* the CUDA-input check by a no-op,

so that ``Operator.integrate`` of a program stepped through its Python callables runs end to end
on the CPU: the integrate driver, the callback plan, the recorders and the output conversions
are the product's own code.
"""

import numpy as np
import torch

from oracle import spectral as S
from torchfsm_gb300 import _lib, _native

_RealSpectral = _native.Spectral


def _library_tables(integrator: int, lin: np.ndarray, dt: float, m: int, r: float) -> list:
    """The scheme's tables in the library's order (oracle values, FP64)."""
    if integrator in (_lib.FSM_ETDRK0, _lib.FSM_ETDRK1, _lib.FSM_ETDRK2):
        order = {_lib.FSM_ETDRK0: 0, _lib.FSM_ETDRK1: 1, _lib.FSM_ETDRK2: 2}[integrator]
        t = S.etdrk_coefs(order, lin, dt)
        keys = ["E", "c1", "c2"][: order + 1]
    else:
        order = {_lib.FSM_SETDRK1: 1, _lib.FSM_SETDRK2: 2, _lib.FSM_SETDRK3: 3, _lib.FSM_SETDRK4: 4}[integrator]
        t = S.setdrk_coefs(order, lin, dt, m, r)
        keys = {1: ["E", "c1"], 2: ["E", "c1", "c2"], 3: ["E", "E2", "c1", "c2", "c3", "c4", "c5"],
                4: ["E", "E2", "c1", "c4", "c5", "c6"]}[order]
    # the exponential tables are stored as E - 1 (the library's layout)
    return [np.broadcast_to(np.asarray(t[k], dtype=np.complex128) - (1.0 if k in ("E", "E2") else 0.0), lin.shape)
            for k in keys]


class _CpuLinearPlan:
    """Stands in for the library plan of a linear part (same constructor as NativePlan)."""

    def __init__(self, program, dt, integrator, device, n_integration_points=16, integration_radius=1.0,
                 linear_coef64=None, table_batch=0):
        assert program.nonlinear == _lib.FSM_NL_NONE and not program.sources
        self.program, self.dt, self.integrator = program, float(dt), integrator
        self.device = torch.device(device)
        self.shape = program.shape
        self.n_channel = program.n_channel
        self.handle = None
        nd = len(self.shape)
        h = self.shape[-1] // 2 + 1
        if linear_coef64 is None:
            lin = np.zeros((1, 1) + self.shape[:-1] + (h,), dtype=np.complex128)
        else:
            L = linear_coef64
            if L.dim() != nd + 2:
                L = L.reshape((1, 1) + tuple(L.shape[-nd:]))
            L = L.expand(tuple(L.shape[:2]) + self.shape)
            lin = L[..., :h].cpu().numpy().astype(np.complex128)
        self.lin_batch = lin.shape[0]
        self._tables = np.stack([t.reshape(-1) for t in _library_tables(
            integrator, lin, self.dt, n_integration_points, integration_radius)])

        self._lin_shape = lin.shape

    def tables(self):
        return torch.from_numpy(self._tables.astype(np.complex64))

    def integrate_half(self, state, steps, slots=None, traj=None, workspace=None):
        """Linear programs (ETDRK0): every point advances by E per step, as the pointwise kernel."""
        if self.integrator != _lib.FSM_ETDRK0:
            raise NotImplementedError("the CPU stand-in steps linear ETDRK0 programs only")
        Em1 = self.tables()[0].reshape(self._lin_shape)
        for i in range(steps):
            if slots is not None and slots[i] >= 0:
                traj[:, slots[i]] = state
            state.add_(Em1 * state)
        if slots is not None and slots[steps] >= 0:
            traj[:, slots[steps]] = state


class _CpuSpectral(_RealSpectral):
    """torch's real FFTs in place of the library's transforms."""

    def to_half(self, u):
        nd = len(self.shape)
        return torch.fft.rfftn(u.to(torch.float32), dim=tuple(range(-nd, 0))).to(torch.complex64)

    def to_physical(self, half, keep_input=True):
        nd = len(self.shape)
        return torch.fft.irfftn(half, s=self.shape, dim=tuple(range(-nd, 0))).to(torch.float32)


def install(monkeypatch):
    monkeypatch.setattr(_native, "NativePlan", _CpuLinearPlan)
    monkeypatch.setattr(_native, "Spectral", _CpuSpectral)
    monkeypatch.setattr(_native, "_require_cuda", lambda t, what: None)


def force_callback(monkeypatch):
    """``install`` plus a lowering that refuses every nonlinear term, so that every nonlinear
    program steps through the callback path (the fused programs included)."""
    install(monkeypatch)
    lower = _native.lower

    def refuse_nonlinear(linear_terms, nonlinear_terms, *args, **kw):
        if nonlinear_terms:
            raise _lib.UnsupportedProgram(_lib.FSM_ERR_UNSUPPORTED, "forced onto the callback path")
        return lower(linear_terms, nonlinear_terms, *args, **kw)

    monkeypatch.setattr(_native, "lower", refuse_nonlinear)

