"""Operator algebra and runtime with the reference's interface (torchfsm/operator/_base.py).

Operators are symbolic sums of (coefficient, core generator). Registering a
mesh turns each generator into a core: a ``LinearCoef`` (a spectral symbol)
or a ``NonlinearFunc`` (a function of the spectrum). ``integrate`` lowers
the cores to a spectral program and runs it in the CUDA library
(``torchfsm_gb300._native``): one fused launch sequence for all steps, the
recorder's frames written by the kernels. ``__call__`` and ``solve``
evaluate the operator once with torch tensor arithmetic.
"""

from __future__ import annotations

import os
from abc import ABC, abstractmethod
from typing import Callable, List, Optional, Sequence, Tuple, Union

import torch
from torch import Tensor

from .. import _lib, _native
from ..integrator import ETDRKIntegrator, RKIntegrator, SETDRKIntegrator
from ..integrator._callback import CALLBACK_SCHEMES, CallbackPlan
from ..mesh import FourierMesh, MeshGrid
from ..traj_recorder import DiskRecorder, RandomBatchWisedRecorder, _TrajRecorder
from ..utils import default

MeshLike = Union[Sequence[Tuple[float, float, int]], MeshGrid, FourierMesh]


class LinearCoef(ABC):
    """A linear spectral symbol (operator/_base.py:16-55)."""

    @abstractmethod
    def __call__(self, f_mesh: FourierMesh, n_channel: int) -> Tensor:
        raise NotImplementedError

    def nonlinear_like(self, u_fft: Tensor, f_mesh: FourierMesh, u: Optional[Tensor] = None) -> Tensor:
        return self(f_mesh, u_fft.shape[1]) * u_fft


class NonlinearFunc(ABC):
    """A nonlinear function of the spectrum (operator/_base.py:58-109).

    ``dealiasing_swtich`` (reference spelling): when True the integrator
    passes the 2/3-masked spectrum and its physical field.
    """

    def __init__(self, dealiasing_swtich: bool = True) -> None:
        self._dealiasing_swtich = dealiasing_swtich

    @abstractmethod
    def __call__(self, u_fft: Tensor, f_mesh: FourierMesh, u: Optional[Tensor] = None) -> Tensor:
        raise NotImplementedError

    def spatial_value(self, u_fft: Tensor, f_mesh: FourierMesh, u: Optional[Tensor] = None) -> Tensor:
        return f_mesh.ifft(self(u_fft, f_mesh, u)).real


class CoreGenerator(ABC):
    """Builds a core from the mesh and the channel count (operator/_base.py:112-131)."""

    @abstractmethod
    def __call__(self, f_mesh: FourierMesh, n_channel: int) -> Union[LinearCoef, NonlinearFunc]:
        raise NotImplementedError


GeneratorLike = Union[CoreGenerator, Callable[[FourierMesh, int], Union[LinearCoef, NonlinearFunc]]]


def check_value_with_mesh(u: Tensor, mesh: MeshLike):
    """Raise ValueError if u [B, C, n1..] does not match the mesh (operator/_base.py:144-167)."""
    if isinstance(mesh, (FourierMesh, MeshGrid)):
        mesh = mesh.mesh_info
    if u.dim() - 2 != len(mesh):
        raise ValueError(f"the value shape {tuple(u.shape)} is not compatible with mesh dim {len(mesh)}")
    for i, m in enumerate(mesh):
        if u.shape[i + 2] != m[2]:
            raise ValueError(f"Expect to have {m[2]} points in dim {i} but got {u.shape[i + 2]}")


class _MutableMixIn:
    """Arithmetic in terms of + and scalar * (operator/_base.py:170-206)."""

    def __radd__(self, other):
        return self + other

    def __iadd__(self, other):
        return self + other

    def __sub__(self, other):
        try:
            return self + (-1 * other)
        except Exception:
            return NotImplemented

    def __rsub__(self, other):
        try:
            return other + (-1 * self)
        except Exception:
            return NotImplemented

    def __isub__(self, other):
        return self - other

    def __rmul__(self, other):
        return self * other

    def __imul__(self, other):
        return self * other

    def __truediv__(self, other):
        try:
            return self * (1 / other)
        except Exception:
            return NotImplemented


class _InverseSolveMixin:
    """Solve L x = b for a linear operator (operator/_base.py:209-262)."""

    def solve(self, b: Optional[Tensor] = None, b_fft: Optional[Tensor] = None, mesh: Optional[MeshLike] = None,
              n_channel: Optional[int] = None, return_in_fourier: bool = False) -> Tensor:
        if not (mesh is not None and n_channel is not None):
            assert self._state_dict["f_mesh"] is not None, "Mesh and n_channel should be given when calling solve"
        if not (mesh is None and n_channel is None):
            mesh = self._state_dict["f_mesh"] if mesh is None else mesh
            n_channel = self._state_dict["n_channel"] if n_channel is None else n_channel
            src = b if b is not None else b_fft
            # a mesh given as a list is registered on the right-hand side's device
            self.register_mesh(mesh, n_channel, device=None if isinstance(mesh, FourierMesh) else src.device)
        if self._state_dict["invert_linear_coef"] is None:
            lin = self.linear_coef
            self._state_dict["invert_linear_coef"] = torch.where(lin == 0, 1.0, 1 / lin)
        f_mesh = self._state_dict["f_mesh"]
        if b_fft is None:
            b_fft = f_mesh.fft(b)
        value_fft = b_fft * self._state_dict["invert_linear_coef"]
        return value_fft if return_in_fourier else f_mesh.ifft(value_fft).real


class _DeAliasMixin:
    """set_de_aliasing_rate (operator/_base.py:265-281)."""

    def set_de_aliasing_rate(self, de_aliasing_rate: float):
        self._de_aliasing_rate = de_aliasing_rate
        self._reset_state()


class NativeETDIntegrator:
    """The integrator object of a registered operator: a library plan for one dt.

    Keeps the reference's integrator protocol (``dt``, ``step(u_hat)``,
    ``forward(u_hat, dt)``) on full spectra; ``integrate`` uses the fused
    multi-step entry point instead.
    """

    def __init__(self, plan: _native.NativePlan):
        self.plan = plan
        self.dt = plan.dt
        self.spectral = _native.Spectral(plan)

    def step(self, u_hat: Tensor) -> Tensor:
        half = self.spectral.full_to_half(u_hat)
        self.plan.integrate_half(half, 1)
        return self.spectral.half_to_full(half).to(u_hat.dtype)

    def forward(self, u_hat: Tensor, dt: float) -> Tensor:
        return self.step(u_hat)


class OperatorLike(_MutableMixIn):
    """Base of all operators (operator/_base.py:284-805)."""

    def __init__(self, operator_generators: Optional[Union[GeneratorLike, List[GeneratorLike]]] = None,
                 coefs: Optional[List] = None) -> None:
        super().__init__()
        self.operator_generators = default(operator_generators, [])
        if not isinstance(self.operator_generators, list):
            self.operator_generators = [self.operator_generators]
        self.coefs = default(coefs, [1] * len(self.operator_generators))
        self._state_dict = None
        self._de_aliasing_rate = 2 / 3
        self._value_mesh_check_func = lambda dim_value, dim_mesh: True
        self._integrator = "auto"
        self._integrator_config = {}
        self._is_etdrk_integrator = True
        self._reset_state()

    def _reset_state(self):
        self._state_dict = {
            "f_mesh": None,
            "n_channel": None,
            "linear_coef": None,
            "nonlinear_func": None,
            "operator": None,
            "integrator": None,
            "invert_linear_coef": None,
            "apply_plan": None,  # library plan of the one-shot evaluation (FSM_APPLY), False if not lowerable
        }
        self._linear_terms = []
        self._nonlinear_funcs = []

    # -- mesh registration -------------------------------------------------
    @property
    def is_linear(self) -> bool:
        assert self._state_dict["f_mesh"] is not None, "Mesh should be registered before checking if the operator is linear"
        return len(self._nonlinear_funcs) == 0 and len(self._linear_terms) > 0

    @property
    def linear_coef(self) -> Optional[Tensor]:
        """L = sum coef * symbol in the mesh dtype (operator/_base.py:339-357), built on first use."""
        if self._state_dict["linear_coef"] is None and self._linear_terms:
            f_mesh, C = self._state_dict["f_mesh"], self._state_dict["n_channel"]
            self._state_dict["linear_coef"] = sum(coef * op(f_mesh, C) for coef, op in self._linear_terms)
        return self._state_dict["linear_coef"]

    def _linear_coef64(self, device) -> Optional[Tensor]:
        """L evaluated on a float64 copy of the registered mesh (input of the FP64 coefficient kernel)."""
        if not self._linear_terms:
            return None
        f_mesh = self._state_dict["f_mesh"]
        fm64 = FourierMesh(f_mesh.mesh_info, device=device, dtype=torch.float64)
        C = self._state_dict["n_channel"]
        total = None
        for coef, op in self._linear_terms:
            if isinstance(coef, Tensor):
                coef = coef.to(device=device, dtype=torch.float64)
            term = coef * op(fm64, C)
            total = term if total is None else total + term
        return total

    def _pre_check(self, u: Optional[Tensor] = None, u_fft: Optional[Tensor] = None,
                   mesh: Optional[MeshLike] = None) -> Tuple[FourierMesh, int]:
        """Shape/device checks; builds a FourierMesh in the value's dtype (operator/_base.py:528-579)."""
        if u_fft is None and u is None:
            raise ValueError("Either u or u_fft should be given")
        if u_fft is not None and u is not None:
            assert u.shape == u_fft.shape, "The shape of u and u_fft should be the same"
        assert mesh is not None, "Mesh should be given"
        value = u if u is not None else u_fft
        value_dtype = value.dtype if not value.is_complex() else value.real.dtype
        if not isinstance(mesh, FourierMesh):
            if not isinstance(mesh, MeshGrid):
                mesh = FourierMesh(mesh, device=value.device, dtype=value_dtype)
            else:
                mesh = FourierMesh(mesh)
        n_channel = value.shape[1]
        assert value.dim() == mesh.n_dim + 2, \
            f"the value shape {tuple(value.shape)} is not compatible with mesh dim {mesh.n_dim}"
        for i in range(mesh.n_dim):
            assert value.shape[i + 2] == mesh.mesh_info[i][2], \
                f"Expect to have {mesh.mesh_info[i][2]} points in dim {i} but got {value.shape[i + 2]}"
        assert value.device == mesh.device, \
            f"The device of mesh {mesh.device} and the device of value {value.device} are not the same"
        assert self._value_mesh_check_func(value.dim() - 2, mesh.n_dim), "Value and mesh do not match the requirement"
        return mesh, n_channel

    def register_mesh(self, mesh: MeshLike, n_channel: int, device=None, dtype=None):
        """Register the mesh and channel count; builds the cores (operator/_base.py:581-624)."""
        if isinstance(mesh, FourierMesh):
            f_mesh = mesh
            if device is not None or dtype is not None:
                f_mesh.to(device=device, dtype=dtype)
        else:
            f_mesh = FourierMesh(mesh, device=device, dtype=dtype)
        self._reset_state()
        self._state_dict["f_mesh"] = f_mesh
        self._state_dict["n_channel"] = n_channel
        for coef, generator in zip(self.coefs, self.operator_generators):
            op = generator(f_mesh, n_channel)
            if isinstance(op, LinearCoef):
                self._linear_terms.append((coef, op))
            elif isinstance(op, NonlinearFunc):
                self._nonlinear_funcs.append((coef, op))
            else:
                raise ValueError(f"Operator {op} is not supported")
        if self._nonlinear_funcs:
            f_mesh.set_default_rel_freq_threshold(self._de_aliasing_rate)
            self._state_dict["nonlinear_func"] = self._nonlinear_closure()

    def _nonlinear_closure(self):
        """Dealiased sum of the nonlinear cores with torch arithmetic (operator/_base.py:375-403),
        used by ``__call__``."""
        funcs = list(self._nonlinear_funcs)

        def nonlinear_funcs_all(u_fft):
            f_mesh = self._state_dict["f_mesh"]
            result = 0.0
            d_fft = d_u = u = None
            for coef, fun in funcs:
                if fun._dealiasing_swtich:
                    if d_fft is None:
                        d_fft = u_fft * f_mesh.low_pass_filter(self._de_aliasing_rate)
                        d_u = f_mesh.ifft(d_fft).real
                    result = result + coef * fun(d_fft, f_mesh, d_u)
                else:
                    if u is None:
                        u = f_mesh.ifft(u_fft).real
                    result = result + coef * fun(u_fft, f_mesh, u)
            return result

        return nonlinear_funcs_all

    def register_additional_check(self, func: Callable[[int, int], bool]):
        self._value_mesh_check_func = func

    def add_generator(self, generator: GeneratorLike, coef=1):
        self.operator_generators.append(generator)
        self.coefs.append(coef)

    def set_integrator(self, integrator, **integrator_config):
        """"auto", an ETDRKIntegrator, SETDRKIntegrator or RKIntegrator member (operator/_base.py:646-674)."""
        if isinstance(integrator, str):
            assert integrator == "auto", \
                "The integrator should be 'auto' or an instance of ETDRKIntegrator, SETDRKIntegrator or RKIntegrator"
        else:
            assert isinstance(integrator, (ETDRKIntegrator, SETDRKIntegrator, RKIntegrator)), \
                "The integrator should be 'auto' or an instance of ETDRKIntegrator, SETDRKIntegrator or RKIntegrator"
        self._integrator = integrator
        self._integrator_config = integrator_config
        if self._state_dict is not None:
            self._state_dict["integrator"] = None

    # -- integration -------------------------------------------------------
    def _integrator_id(self) -> int:
        if self._integrator == "auto":
            return _lib.FSM_ETDRK0 if self.is_linear else _lib.FSM_SETDRK4
        if isinstance(self._integrator, RKIntegrator) and self._integrator_config.get("adaptive", False):
            raise NotImplementedError("adaptive step-size control of the Runge-Kutta integrators is not provided "
                                      "by torchfsm_gb300; the fixed-step schemes are")
        return int(self._integrator.value)

    @torch.no_grad()
    def _build_integrator(self, dt: float, device: torch.device):
        if not self._linear_terms and not self._nonlinear_funcs:
            raise ValueError("Both linear coefficient and nonlinear function are None. Cannot build operator.")
        integ = self._integrator_id()
        if integ == _lib.FSM_ETDRK0:
            assert self.is_linear, "The ETDRK0 integrator only supports linear term"
        f_mesh = self._state_dict["f_mesh"]
        callback = False
        try:
            prog = _native.lower(self._linear_terms, self._nonlinear_funcs, f_mesh, self._state_dict["n_channel"],
                                 self._de_aliasing_rate)
        except _lib.UnsupportedProgram as err:
            # nonlinear terms without a fused kernel: the linear part's plan steps them through the
            # cores' Python callables (integrator/_callback.py); anything else stays unsupported
            if not self._nonlinear_funcs:
                raise
            try:
                prog = _native.lower(self._linear_terms, [], f_mesh, self._state_dict["n_channel"],
                                     self._de_aliasing_rate)
            except _lib.UnsupportedProgram:
                raise err from None
            if integ not in CALLBACK_SCHEMES:
                raise _lib.UnsupportedProgram(
                    _lib.FSM_ERR_UNSUPPORTED,
                    f"{err}; such terms step with ETDRK1/2 or SETDRK1-4, not the Runge-Kutta schemes") from None
            callback = True
        cfg = dict(self._integrator_config)
        try:
            plan = _native.NativePlan(
                prog, dt, integ, device,
                n_integration_points=cfg.get("n_integration_points", 16),
                integration_radius=cfg.get("integration_radius", 1.0),
                linear_coef64=self._linear_coef64(device),
            )
        except _lib.FsmError as e:
            if e.code == _lib.FSM_ERR_OOM:
                raise RuntimeError(os.linesep.join([
                    "Cuda out of memory when building the integrator.",
                    f"Original error message: {e}",
                    "Please try to use a smaller mesh or a low-order integrator."])) from e
            raise
        if callback:
            plan = CallbackPlan(plan, self._nonlinear_funcs, f_mesh, self._de_aliasing_rate)
        self._is_etdrk_integrator = True
        self._state_dict["integrator"] = NativeETDIntegrator(plan)

    def integrate(self, u_0: Optional[Tensor] = None, u_0_fft: Optional[Tensor] = None, dt: float = 1, step: int = 1,
                  mesh: Optional[MeshLike] = None, progressive: bool = False,
                  trajectory_recorder: Optional[_TrajRecorder] = None, return_in_fourier: bool = False) -> Tensor:
        """Integrate ``step`` steps of ``dt`` from u_0 (or its spectrum) (operator/_base.py:676-751).

        Returns the final field [B, C, n1..] (real, or the full complex
        spectrum if ``return_in_fourier``), or with a recorder its
        ``trajectory`` [B, T, C, n1..]. Runs in FP32/complex64 on the CUDA
        device of the input. ``progressive`` (the reference's tqdm bar) is
        accepted and has no effect: the steps are enqueued as one launch
        sequence, with no per-step host loop to report on.
        """
        if self._state_dict["f_mesh"] is None or mesh is not None:
            mesh, n_channel = self._pre_check(u=u_0, u_fft=u_0_fft, mesh=mesh)
            self.register_mesh(mesh, n_channel)
        else:
            self._pre_check(u=u_0, u_fft=u_0_fft, mesh=self._state_dict["f_mesh"])
        value = u_0 if u_0 is not None else u_0_fft
        _native._require_cuda(value, "the initial condition")
        device = value.device
        if value.shape[0] == 0:
            return self._empty_integration(value, int(step), trajectory_recorder, return_in_fourier)
        integ = self._state_dict["integrator"]
        if integ is None or integ.dt != dt or integ.plan.device != device:
            self._build_integrator(dt, device)
            integ = self._state_dict["integrator"]
        real_dtype = value.dtype if not value.is_complex() else value.real.dtype
        _native.warn_precision(real_dtype)
        needs_grad = torch.is_grad_enabled() and (
            (u_0 is not None and u_0.requires_grad)
            or any(isinstance(c, Tensor) and c.requires_grad for c, _ in self._linear_terms))
        if needs_grad:
            if trajectory_recorder is not None or return_in_fourier or u_0 is None:
                raise NotImplementedError("gradients are provided for integrate(u_0, ...) returning the final field")
            from ..adjoint import integrate_with_grad

            return integrate_with_grad(self, u_0, dt, int(step)).to(real_dtype)
        sp = integ.spectral
        if u_0_fft is None:
            state = sp.to_half(u_0)
        else:
            state = sp.full_to_half(u_0_fft)
        state = state.contiguous()
        try:
            if trajectory_recorder is None:
                integ.plan.integrate_half(state, int(step))
            elif trajectory_recorder._accepts_blocks():
                sel = [i for i in range(int(step) + 1) if trajectory_recorder.control_func(i)]
                slots = [-1] * (int(step) + 1)
                for j, i in enumerate(sel):
                    slots[i] = j
                traj = None
                if sel:
                    traj = torch.empty((state.shape[0], len(sel)) + tuple(state.shape[1:]),
                                       dtype=torch.complex64, device=device)
                integ.plan.integrate_half(state, int(step), slots=slots, traj=traj)
                if traj is not None:
                    trajectory_recorder._add_block(traj, sp)
            else:
                # custom recorder: keep the per-step protocol on full spectra
                for i in range(int(step)):
                    trajectory_recorder.record(i, sp.half_to_full(state))
                    integ.plan.integrate_half(state, 1)
                trajectory_recorder.record(int(step), sp.half_to_full(state))
        except _lib.FsmError as e:
            if e.code == _lib.FSM_ERR_OOM:
                raise RuntimeError(os.linesep.join([
                    "Cuda out of memory when integrating the operator.",
                    f"Original error message: {e}",
                    "Please try to use a smaller mesh or a low-order integrator."])) from e
            raise
        cplx = torch.complex128 if real_dtype == torch.float64 else torch.complex64
        if trajectory_recorder is not None:
            trajectory_recorder.return_in_fourier = return_in_fourier
            out = trajectory_recorder.trajectory
            if out is not None:
                out = out.to(cplx if return_in_fourier else real_dtype)
            return out
        if return_in_fourier:
            return sp.half_to_full(state).to(cplx)
        return sp.to_physical(state, keep_input=False).to(real_dtype)

    def _empty_integration(self, value: Tensor, step: int, recorder: Optional[_TrajRecorder],
                           return_in_fourier: bool) -> Optional[Tensor]:
        """The result of integrating an empty batch, with nothing launched: [0, C, n..] (or the
        recorder's [0, T, C, n..]) in the dtype the call would return. The reference has no rule
        for this case: its first forward transform raises on a batch of zero samples (MKL on the
        CPU), so empty results are returned here instead of a library error."""
        real_dtype = value.dtype if not value.is_complex() else value.real.dtype
        cplx = torch.complex128 if real_dtype == torch.float64 else torch.complex64
        dtype = cplx if return_in_fourier else real_dtype
        lead = (0, self._state_dict["n_channel"])
        shape = tuple(int(m[2]) for m in self._state_dict["f_mesh"].mesh_info)
        if recorder is None:
            return torch.empty(lead + shape, dtype=dtype, device=value.device)
        recorder.return_in_fourier = return_in_fourier
        if isinstance(recorder, DiskRecorder):
            return None
        if isinstance(recorder, RandomBatchWisedRecorder):
            frames = recorder.n_recorded_frames
        else:
            frames = sum(1 for i in range(step + 1) if recorder.control_func(i))
        return torch.empty((0, frames) + lead[1:] + shape, dtype=dtype, device=value.device)

    # -- one-shot evaluation -----------------------------------------------
    def _build_operator(self):
        lin = self.linear_coef
        nl = self._state_dict["nonlinear_func"]
        if nl is None and lin is None:
            raise ValueError("Both linear coefficient and nonlinear function are None. Cannot build operator.")
        if nl is None:
            op = lambda u_fft: lin * u_fft
        elif lin is None:
            op = lambda u_fft: nl(u_fft)
        else:
            op = lambda u_fft: lin * u_fft + nl(u_fft)
        self._state_dict["operator"] = op

    def __call__(self, u: Optional[Tensor] = None, u_fft: Optional[Tensor] = None, mesh: Optional[MeshLike] = None,
                 return_in_fourier: bool = False) -> Tensor:
        """L u_hat + N(u_hat) once (operator/_base.py:753-790).

        Programs the library lowers (the ones ``integrate`` runs fused) evaluate through the
        fused kernels: a one-step launch sequence of the FSM_APPLY scheme writes the
        right-hand side over a half-spectrum copy of the (real) input; they need CUDA inputs.
        Other programs (channel-changing post-processing cores, Python callables) evaluate their
        cores with torch on the input's device."""
        if self._state_dict["f_mesh"] is None or mesh is not None:
            mesh, n_channel = self._pre_check(u, u_fft, mesh)
            self.register_mesh(mesh, n_channel)
        else:
            self._pre_check(u=u, u_fft=u_fft, mesh=self._state_dict["f_mesh"])
        fused = self._apply_fused(u, u_fft)
        if fused is not None:
            half, sp, dtype = fused
            if return_in_fourier:
                out = sp.half_to_full(half)
                return out.to(torch.complex128) if dtype == torch.float64 else out
            return sp.to_physical(half, keep_input=False).to(dtype)
        if self._state_dict["operator"] is None:
            self._build_operator()
        f_mesh = self._state_dict["f_mesh"]
        if u_fft is None:
            u_fft = f_mesh.fft(u)
        value_fft = self._state_dict["operator"](u_fft)
        return value_fft if return_in_fourier else f_mesh.ifft(value_fft).real

    @torch.no_grad()
    def _apply_fused(self, u: Optional[Tensor], u_fft: Optional[Tensor]):
        """(half spectrum of L u + N(u), its Spectral, the input's real dtype) through the library,
        or None where the program does not lower or the input is not on a CUDA device."""
        src = u if u is not None else u_fft
        if src is None or self._state_dict["apply_plan"] is False:
            return None
        if any(isinstance(c, Tensor) and c.requires_grad for c, _ in self._linear_terms):
            return None  # keep autograd through torch for tensor coefficients that want gradients
        if not src.is_cuda:
            # programs the library covers run only there: no CPU evaluation of them
            try:
                _native.lower(self._linear_terms, self._nonlinear_funcs, self._state_dict["f_mesh"],
                              self._state_dict["n_channel"], self._de_aliasing_rate)
            except _lib.UnsupportedProgram:
                self._state_dict["apply_plan"] = False
                return None
            _native._require_cuda(src, "the operator's input")
        plan = self._state_dict["apply_plan"]
        if plan is None or plan.device != src.device:
            f_mesh = self._state_dict["f_mesh"]
            try:
                prog = _native.lower(self._linear_terms, self._nonlinear_funcs, f_mesh,
                                     self._state_dict["n_channel"], self._de_aliasing_rate)
                plan = _native.NativePlan(prog, 1.0, _lib.FSM_APPLY, src.device,
                                          linear_coef64=self._linear_coef64(src.device))
            except _lib.UnsupportedProgram:
                self._state_dict["apply_plan"] = False
                return None
            self._state_dict["apply_plan"] = plan
        sp = _native.Spectral(plan)
        if u is not None:
            dtype = u.dtype
            half = sp.to_half(u)
        else:
            dtype = torch.float64 if u_fft.dtype == torch.complex128 else torch.float32
            half = sp.full_to_half(u_fft)
        half = half.contiguous()
        plan.integrate_half(half, 1)
        return half, sp, dtype

    def to(self, device=None, dtype=None):
        if self._state_dict["f_mesh"] is not None:
            f_mesh, C = self._state_dict["f_mesh"], self._state_dict["n_channel"]
            f_mesh.to(device=device, dtype=dtype)
            self.register_mesh(f_mesh, C)


class Operator(OperatorLike, _DeAliasMixin):
    """Linear and nonlinear terms (operator/_base.py:807-850)."""

    def __add__(self, other):
        if isinstance(other, OperatorLike):
            return Operator(self.operator_generators + other.operator_generators, self.coefs + other.coefs)
        if isinstance(other, Tensor):
            return Operator(self.operator_generators + [_source_generator(other)], self.coefs + [1])
        return NotImplemented

    def __mul__(self, other):
        if isinstance(other, OperatorLike):
            return NotImplemented
        return Operator(self.operator_generators, [c * other for c in self.coefs])

    def __neg__(self):
        return Operator(self.operator_generators, [-1 * c for c in self.coefs])


def _wrap_cores(items, base):
    out = []
    for it in items:
        if isinstance(it, base):
            out.append((lambda core: (lambda f_mesh, n_channel: core))(it))
        else:
            out.append(it)
    return out


class LinearOperator(OperatorLike, _InverseSolveMixin):
    """Linear terms only (operator/_base.py:853-919)."""

    def __init__(self, linear_coef=None, coefs: Optional[List] = None) -> None:
        if not isinstance(linear_coef, list):
            linear_coef = [linear_coef]
        super().__init__(operator_generators=_wrap_cores(linear_coef, LinearCoef), coefs=coefs)

    @property
    def is_linear(self):
        return True

    def __add__(self, other):
        if isinstance(other, LinearOperator):
            return LinearOperator(self.operator_generators + other.operator_generators, self.coefs + other.coefs)
        if isinstance(other, OperatorLike):
            return Operator(self.operator_generators + other.operator_generators, self.coefs + other.coefs)
        if isinstance(other, Tensor):
            return Operator(self.operator_generators + [_source_generator(other)], self.coefs + [1])
        return NotImplemented

    def __mul__(self, other):
        if isinstance(other, OperatorLike):
            return NotImplemented
        return LinearOperator(self.operator_generators, [c * other for c in self.coefs])

    def __neg__(self):
        return LinearOperator(self.operator_generators, [-1 * c for c in self.coefs])


class NonlinearOperator(OperatorLike, _DeAliasMixin):
    """Nonlinear terms only (operator/_base.py:922-988)."""

    def __init__(self, nonlinear_func=None, coefs: Optional[List] = None) -> None:
        if not isinstance(nonlinear_func, list):
            nonlinear_func = [nonlinear_func]
        super().__init__(operator_generators=_wrap_cores(nonlinear_func, NonlinearFunc), coefs=coefs)

    @property
    def is_linear(self):
        return False

    def __add__(self, other):
        if isinstance(other, NonlinearOperator):
            return NonlinearOperator(self.operator_generators + other.operator_generators, self.coefs + other.coefs)
        if isinstance(other, OperatorLike):
            return Operator(self.operator_generators + other.operator_generators, self.coefs + other.coefs)
        if isinstance(other, Tensor):
            return Operator(self.operator_generators + [_source_generator(other)], self.coefs + [1])
        return NotImplemented

    def __mul__(self, other):
        if isinstance(other, OperatorLike):
            return NotImplemented
        return NonlinearOperator(self.operator_generators, [c * other for c in self.coefs])

    def __neg__(self):
        return NonlinearOperator(self.operator_generators, [-1 * c for c in self.coefs])


class _ExplicitSourceCore(NonlinearFunc):
    """A fixed source field added to the nonlinear value, not dealiased (operator/_base.py:994-1015)."""

    def __init__(self, source: Tensor) -> None:
        super().__init__(dealiasing_swtich=False)
        self.source_physical = source
        self.source = torch.fft.fftn(source, dim=[i + 2 for i in range(source.dim() - 2)])

    def __call__(self, u_fft: Tensor, f_mesh: FourierMesh, u: Optional[Tensor] = None) -> Tensor:
        if self.source.device != f_mesh.device:
            self.source = self.source.to(f_mesh.device)
        return self.source


def _source_generator(source: Tensor):
    core = _ExplicitSourceCore(source)
    return lambda f_mesh, n_channel: core


class ExplicitSource(NonlinearOperator):
    """Explicit source term: ``op + tensor`` (operator/_base.py:1018-1028)."""

    def __init__(self, source: Tensor) -> None:
        super().__init__(_ExplicitSourceCore(source))
