"""Lowering of operators to the CUDA library and the fused integrate entry.

An operator's (coefficient, core) list is lowered to a spectral program:
the linear symbol L = sum coef * symbol evaluated in FP64 (any ``LinearCoef``
works, batched tensor coefficients included), at most one recognised
nonlinear term (Convection, VorticityConvection, KSConvection,
NSPressureConvection without external force) with a scalar coefficient,
explicit sources folded into one spectrum, the per-axis dealias masks and
the integrator. ``NativePlan`` owns the library plan built from it;
``Spectral`` wraps a plan's transforms and the half <-> full spectrum
conversions.
"""

from __future__ import annotations

import ctypes
import math
import warnings
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import torch

from . import _lib

_WARNED_FP64 = False


def _stream(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _require_cuda(t: torch.Tensor, what: str) -> None:
    if not t.is_cuda:
        raise RuntimeError(
            f"torchfsm_gb300 runs on CUDA devices only: {what} is on {t.device}. "
            "Move it to a CUDA device (there is no CPU path)."
        )


@dataclass
class SpectralProgram:
    mesh_info: Tuple[Tuple[float, float, int], ...]
    n_channel: int
    nonlinear: int = _lib.FSM_NL_NONE
    nonlinear_coef: float = 0.0
    flags: int = 0
    linear_terms: List = field(default_factory=list)   # (coef, LinearCoef)
    sources: List = field(default_factory=list)        # (coef, physical source tensor)
    keep: Optional[List[torch.Tensor]] = None          # per-axis uint8 masks
    has_nonlinear: bool = False

    @property
    def ndim(self) -> int:
        return len(self.mesh_info)

    @property
    def shape(self) -> Tuple[int, ...]:
        return tuple(int(m[2]) for m in self.mesh_info)


def lower(linear_terms, nonlinear_terms, f_mesh, n_channel: int, de_aliasing_rate: float) -> SpectralProgram:
    """Build the spectral program of an operator, or raise UnsupportedProgram."""
    from .operator import _base as B
    from .operator.dedicated._ks_convection import _KSConvectionCore
    from .operator.dedicated._navier_stokes import _NSPressureConvectionCore, _VorticityConvectionCore
    from .operator.generic._convection import _ConvectionCore

    prog = SpectralProgram(tuple(tuple(m) for m in f_mesh.mesh_info), n_channel)
    for _, fun in linear_terms:
        sym = fun(f_mesh, n_channel)
        if isinstance(sym, torch.Tensor) and sym.dim() >= 2 and sym.shape[1] not in (1, n_channel):
            raise _lib.UnsupportedProgram(_lib.FSM_ERR_UNSUPPORTED, "a linear term that changes the channel count")
    prog.linear_terms = list(linear_terms)
    kinds = {}
    for coef, fun in nonlinear_terms:
        prog.has_nonlinear = True
        if isinstance(fun, B._ExplicitSourceCore):
            prog.sources.append((coef, fun.source_physical))
            continue
        if isinstance(fun, _ConvectionCore) and type(fun) is _ConvectionCore:
            key = (_lib.FSM_NL_CONVECTION, 0)
        elif isinstance(fun, _VorticityConvectionCore):
            key = (_lib.FSM_NL_VORTICITY, 0)
        elif isinstance(fun, _KSConvectionCore):
            key = (_lib.FSM_NL_KS, _lib.FSM_FLAG_REMOVE_MEAN if fun.remove_mean else 0)
        elif isinstance(fun, _NSPressureConvectionCore) and fun.external_force is None:
            key = (_lib.FSM_NL_LERAY, 0)
        else:
            raise _lib.UnsupportedProgram(_lib.FSM_ERR_UNSUPPORTED,
                                          f"no fused kernel for the nonlinear term {type(fun).__name__}")
        if not getattr(fun, "_dealiasing_swtich", True):
            raise _lib.UnsupportedProgram(_lib.FSM_ERR_UNSUPPORTED, "non-dealiased nonlinear terms")
        if isinstance(coef, torch.Tensor):
            if coef.numel() != 1:
                raise _lib.UnsupportedProgram(_lib.FSM_ERR_UNSUPPORTED, "tensor coefficient on a nonlinear term")
            coef = float(coef.item())
        kinds[key] = kinds.get(key, 0.0) + float(coef)
    if len(kinds) > 1:
        raise _lib.UnsupportedProgram(_lib.FSM_ERR_UNSUPPORTED, "more than one kind of nonlinear term")
    if kinds:
        (kind, flags), coef = next(iter(kinds.items()))
        prog.nonlinear, prog.flags, prog.nonlinear_coef = kind, flags, coef
    prog.keep = f_mesh.axis_keep(de_aliasing_rate)
    return prog


class Spectral:
    """Transforms between physical fields and half spectra on one mesh."""

    def __init__(self, plan: "NativePlan"):
        self.plan = plan
        self.shape = plan.shape
        self.device = plan.device

    @property
    def half_last(self) -> int:
        return self.shape[-1] // 2 + 1

    def to_half(self, u: torch.Tensor) -> torch.Tensor:
        """Real [.., n1..nd] -> half spectra [.., n1.., nd/2+1] (complex64)."""
        nd = len(self.shape)
        lead = u.shape[: u.dim() - nd]
        x = u.to(device=self.device, dtype=torch.float32).contiguous()
        count = int(math.prod(lead)) if lead else 1
        out = torch.empty(tuple(lead) + self.shape[:-1] + (self.half_last,), dtype=torch.complex64, device=self.device)
        _lib.check(_lib.load().fsm_rfftn(self.plan.handle, count, x.data_ptr(), out.data_ptr(), _stream(self.device)))
        return out

    def to_physical(self, half: torch.Tensor, keep_input: bool = True) -> torch.Tensor:
        """Half spectra -> real fields (= ifftn(full).real)."""
        nd = len(self.shape)
        lead = half.shape[: half.dim() - nd]
        src = half.contiguous()
        if keep_input and src.data_ptr() == half.data_ptr():
            src = src.clone()
        count = int(math.prod(lead)) if lead else 1
        out = torch.empty(tuple(lead) + self.shape, dtype=torch.float32, device=self.device)
        _lib.check(_lib.load().fsm_irfftn(self.plan.handle, count, src.data_ptr(), out.data_ptr(), _stream(self.device)))
        return out

    def half_to_full(self, half: torch.Tensor) -> torch.Tensor:
        """Hermitian extension of half spectra to the full complex spectrum."""
        nd = len(self.shape)
        n = self.shape[-1]
        h = self.half_last
        full = torch.empty(half.shape[:-1] + (n,), dtype=half.dtype, device=half.device)
        full[..., :h] = half
        if n > 2:
            m = half[..., 1 : n - h + 1].conj()
            for ax in range(half.dim() - nd, half.dim() - 1):
                m = torch.roll(torch.flip(m, dims=[ax]), shifts=1, dims=[ax])
            full[..., h:] = torch.flip(m, dims=[-1])
        return full

    def full_to_half(self, full: torch.Tensor) -> torch.Tensor:
        """Half spectrum of the real part of ifftn(full): (F(k) + conj F(-k)) / 2 on the kept half."""
        nd = len(self.shape)
        f = full.to(device=self.device, dtype=torch.complex64)
        m = f.conj()
        for ax in range(f.dim() - nd, f.dim()):
            m = torch.roll(torch.flip(m, dims=[ax]), shifts=1, dims=[ax])
        return (0.5 * (f + m))[..., : self.half_last].contiguous()


class NativePlan:
    """A library plan for one (program, mesh, dt) on one device."""

    def __init__(self, program: SpectralProgram, dt: float, integrator: int, device: torch.device,
                 n_integration_points: int = 16, integration_radius: float = 1.0,
                 linear_coef64: Optional[torch.Tensor] = None, table_batch: int = 0):
        self.program = program
        self.dt = float(dt)
        self.integrator = integrator
        self.device = device
        self.shape = program.shape
        self.n_channel = program.n_channel
        self.handle = None
        lib = _lib.load()
        nd = program.ndim
        mesh = _lib.FsmMeshDesc()
        mesh.ndim = nd
        for i, (s, e, n) in enumerate(program.mesh_info):
            mesh.n[i] = int(n)
            mesh.length[i] = float(e - s)
        desc = _lib.FsmProgramDesc()
        desc.n_channel = program.n_channel
        desc.nonlinear = program.nonlinear
        desc.flags = program.flags
        desc.integrator = integrator
        desc.nonlinear_coef = program.nonlinear_coef
        keep_bufs = []
        for i in range(nd):
            kb = (ctypes.c_uint8 * len(program.keep[i]))(*[int(v) for v in program.keep[i].tolist()])
            keep_bufs.append(kb)
            desc.keep[i] = ctypes.cast(kb, ctypes.c_void_p)
        desc.n_integration_points = int(n_integration_points)
        desc.integration_radius = float(integration_radius)
        self._lin_half = None
        self.lin_batch = 1
        if linear_coef64 is not None:
            lin = linear_coef64
            C = program.n_channel
            full = lin.shape
            lb = full[0] if lin.dim() == nd + 2 else 1
            lc = full[1] if lin.dim() == nd + 2 else 1
            lin = lin.reshape((lb, lc) + tuple(lin.shape[-nd:])) if lin.dim() != nd + 2 else lin
            lin = lin.expand((lb, lc) + self.shape)
            if lc not in (1, C):
                raise _lib.FsmError(_lib.FSM_ERR_INVALID, f"linear coefficient with {lc} channels for {C}")
            h = self.shape[-1] // 2 + 1
            half = lin[..., :h].to(device=device, dtype=torch.complex128).contiguous()
            self._lin_half = half
            self.lin_batch = lb
            desc.linear_coef = half.data_ptr()
            desc.lin_batch = lb
            desc.lin_channel = lc
        else:
            desc.lin_batch = 1
            desc.lin_channel = 1
        desc.table_batch = int(table_batch)
        self.table_batch = int(table_batch)
        self.src_batch = 0
        self._src_half = None
        handle = ctypes.c_void_p()
        stream = _stream(device)
        if program.sources:
            # transforms only need the mesh: a bare plan turns the sources into spectra
            bare = NativePlan.__new__(NativePlan)
            bare.__init__(SpectralProgram(program.mesh_info, program.n_channel, keep=program.keep), dt,
                          _lib.FSM_ETDRK0, device)
            sp = Spectral(bare)
            total = None
            for coef, src in program.sources:
                s = src.to(device)
                while s.dim() < nd + 2:
                    s = s.unsqueeze(0)
                part = sp.to_half(s.expand((s.shape[0], program.n_channel) + self.shape))
                part = part * complex(coef) if not isinstance(coef, torch.Tensor) else part * coef.to(device)
                total = part if total is None else total + part
            self._src_half = total.to(torch.complex64).contiguous()
            self.src_batch = self._src_half.shape[0]
            desc.source = self._src_half.data_ptr()
            desc.src_batch = self.src_batch
        _lib.check(lib.fsm_plan_create(ctypes.byref(mesh), ctypes.byref(desc), float(dt), stream, ctypes.byref(handle)))
        self.handle = handle
        self._lin_half = None  # consumed by the plan (stream synchronised in fsm_plan_create)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _lib.load().fsm_plan_destroy(h)
            except Exception:
                pass
            self.handle = None

    def tables(self) -> torch.Tensor:
        """The plan's coefficient tables [ntab, table_batch * lin_channel * S] (complex64)."""
        lib = _lib.load()
        nt, ne = ctypes.c_int32(), ctypes.c_int64()
        _lib.check(lib.fsm_plan_tables(self.handle, None, 0, ctypes.byref(nt), ctypes.byref(ne), None))
        out = torch.empty((nt.value, ne.value), dtype=torch.complex64, device=self.device)
        _lib.check(lib.fsm_plan_tables(self.handle, out.data_ptr(), out.numel() * 8, None, None,
                                       _stream(self.device)))
        return out

    def set_batch_dt(self, b: int, dt: float) -> None:
        """Recompute the tables of batch entry b for time step dt (plans built with table_batch > 1)."""
        _lib.check(_lib.load().fsm_plan_set_batch_dt(self.handle, int(b), float(dt), _stream(self.device)))

    def move_batch(self, dst: int, src: int) -> None:
        """Copy the tables of batch entry src to entry dst."""
        _lib.check(_lib.load().fsm_plan_move_batch(self.handle, int(dst), int(src), _stream(self.device)))

    def workspace_bytes(self, batch: int, steps: int) -> int:
        out = ctypes.c_size_t()
        _lib.check(_lib.load().fsm_plan_workspace_bytes(self.handle, batch, steps, ctypes.byref(out)))
        return int(out.value)

    def launch_count(self, steps: int, batch: int = 0) -> int:
        out = ctypes.c_int64()
        _lib.check(_lib.load().fsm_plan_launch_count(self.handle, batch, steps, ctypes.byref(out)))
        return int(out.value)

    def integrate_half(self, state: torch.Tensor, steps: int, slots: Optional[Sequence[int]] = None,
                       traj: Optional[torch.Tensor] = None, workspace: Optional[torch.Tensor] = None) -> None:
        """Advance half spectra [B, C, S] (complex64, contiguous, in place)."""
        B = state.shape[0]
        need = self.workspace_bytes(B, steps)
        if workspace is None or workspace.numel() < need:
            workspace = torch.empty(need, dtype=torch.uint8, device=self.device)
        slot_arr = None
        n_frames = 0
        if slots is not None:
            slot_arr = (ctypes.c_int32 * (steps + 1))(*slots)
            n_frames = traj.shape[1] if traj is not None else 0
        _lib.check(_lib.load().fsm_integrate(
            self.handle, B, state.data_ptr(), steps,
            ctypes.cast(slot_arr, ctypes.c_void_p) if slot_arr is not None else None,
            traj.data_ptr() if traj is not None else None, n_frames,
            workspace.data_ptr(), need, _stream(self.device)))


class ServePool:
    """The library's serving engine (``fsm_serve_*``) over one plan built with
    ``table_batch >= capacity``: requests of half-spectrum samples are queued, admitted into
    slots at tick boundaries, advanced together and written back in place when their steps
    are done. All work runs on ``stream``; the state and workspace tensors are kept alive here."""

    STATS = ("occupied", "waiting", "active", "in_flight", "ticks", "launches", "graph_replays",
             "slot_steps", "completed", "cancelled")

    def __init__(self, plan: NativePlan, capacity: int, chunk: int, stream: torch.cuda.Stream,
                 graphs: bool = True, tick_ms: float = 0.0):
        self.plan = plan
        self.capacity, self.chunk = int(capacity), int(chunk)
        self.stream = stream
        shape = plan.shape
        half = tuple(shape[:-1]) + (shape[-1] // 2 + 1,)
        self.sample_shape = (plan.n_channel,) + half
        self.handle = None
        with torch.cuda.stream(stream):
            self.state = torch.empty((self.capacity,) + self.sample_shape, dtype=torch.complex64, device=plan.device)
            need = ctypes.c_size_t()
            _lib.check(_lib.load().fsm_serve_workspace_bytes(plan.handle, self.capacity, self.chunk,
                                                             ctypes.byref(need)))
            self.ws = torch.empty(need.value, dtype=torch.uint8, device=plan.device)
        handle = ctypes.c_void_p()
        _lib.check(_lib.load().fsm_serve_create(
            plan.handle, self.capacity, self.chunk, self.state.data_ptr(), self.ws.data_ptr(), self.ws.numel(),
            _lib.FSM_SERVE_GRAPHS if graphs else 0, float(tick_ms), stream.cuda_stream, ctypes.byref(handle)))
        self.handle = handle
        self._ids = (ctypes.c_int64 * 256)()

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _lib.load().fsm_serve_destroy(h)
            except Exception:
                pass
            self.handle = None

    def submit(self, rid: int, steps: int, dt: float, half: torch.Tensor) -> None:
        """Queue ``half`` ([batch, C, ...] complex64 half spectra on the pool's device, written
        stream-ordered on the pool's stream) for ``steps`` steps of ``dt``; the result replaces it."""
        _require_cuda(half, "serve input")
        if tuple(half.shape[1:]) != self.sample_shape or half.dtype != torch.complex64 or not half.is_contiguous():
            raise _lib.FsmError(_lib.FSM_ERR_INVALID, f"serve input {tuple(half.shape)} for samples {self.sample_shape}")
        _lib.check(_lib.load().fsm_serve_submit(self.handle, int(rid), half.shape[0], int(steps), float(dt),
                                                half.data_ptr(), half.data_ptr()))

    def tick(self) -> int:
        """Admit what fits and launch the next tick; the steps launched (0: busy or idle)."""
        k = ctypes.c_int32()
        _lib.check(_lib.load().fsm_serve_tick(self.handle, ctypes.byref(k)))
        return int(k.value)

    def poll(self, wait: bool = False) -> Tuple[List[int], bool]:
        """Complete the tick in flight if it is done (or wait for it): (completed ids, tick in flight)."""
        lib = _lib.load()
        ids: List[int] = []
        n, busy = ctypes.c_int32(), ctypes.c_int32()
        while True:
            _lib.check(lib.fsm_serve_poll(self.handle, 1 if wait else 0, self._ids, len(self._ids), ctypes.byref(n),
                                          ctypes.byref(busy)))
            ids.extend(self._ids[i] for i in range(n.value))
            if n.value < len(self._ids):
                return ids, bool(busy.value)
            wait = False

    def cancel(self, rid: int) -> None:
        _lib.check(_lib.load().fsm_serve_cancel(self.handle, int(rid)))

    def status(self, rid: int) -> Tuple[int, int]:
        st, rem = ctypes.c_int32(), ctypes.c_int32()
        _lib.check(_lib.load().fsm_serve_request_status(self.handle, int(rid), ctypes.byref(st), ctypes.byref(rem)))
        return int(st.value), int(rem.value)

    def stats(self) -> dict:
        arr = (ctypes.c_int64 * len(self.STATS))()
        _lib.check(_lib.load().fsm_serve_stats(self.handle, arr, len(self.STATS)))
        return dict(zip(self.STATS, list(arr)))


class ServeGroup:
    """Serving engines of different grid sizes ticked together (``fsm_serve_group_*``): one tick
    advances every occupied slot of every member by the same number of steps: as ONE kernel
    launch when every member is a 1D line plan of one nonlinear kind, with one launch per pass
    when every member is a square 2D plan (64, 128, 256) of one nonlinear kind, else the members
    one after the other. The members share one stream; requests are still submitted to and polled from
    them. Close the group before its members."""

    STATS = ("ticks", "launches", "in_flight", "one_launch", "one_launch_per_pass")

    def __init__(self, pools: List[ServePool], tick_ms: float = 0.0):
        self.pools = list(pools)
        self.handle = None
        arr = (ctypes.c_void_p * len(self.pools))(*[p.handle.value for p in self.pools])
        handle = ctypes.c_void_p()
        _lib.check(_lib.load().fsm_serve_group_create(arr, len(self.pools), float(tick_ms), ctypes.byref(handle)))
        self.handle = handle

    def close(self) -> None:
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self.handle = None
            _lib.check(_lib.load().fsm_serve_group_destroy(h))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tick(self) -> int:
        """Admit into every member and launch the group's next tick; the steps launched (0: busy or idle)."""
        k = ctypes.c_int32()
        _lib.check(_lib.load().fsm_serve_group_tick(self.handle, ctypes.byref(k)))
        return int(k.value)

    def poll(self, wait: bool = False) -> bool:
        """Complete the group's tick if it is done (or wait for it); whether a tick is still in flight.
        The members' completed ids are then read with their ``poll``."""
        busy = ctypes.c_int32()
        _lib.check(_lib.load().fsm_serve_group_poll(self.handle, 1 if wait else 0, ctypes.byref(busy)))
        return bool(busy.value)

    def stats(self) -> dict:
        arr = (ctypes.c_int64 * len(self.STATS))()
        _lib.check(_lib.load().fsm_serve_group_stats(self.handle, arr, len(self.STATS)))
        return dict(zip(self.STATS, list(arr)))


def warn_precision(dtype: torch.dtype) -> None:
    global _WARNED_FP64
    if dtype == torch.float64 and not _WARNED_FP64:
        warnings.warn("torchfsm_gb300 integrates in FP32/complex64; float64 inputs are rounded and the "
                      "result is returned in float64", stacklevel=3)
        _WARNED_FP64 = True
