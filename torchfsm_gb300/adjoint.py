"""Hand-written adjoint of the fused SETDRK4 integration (gradients w.r.t. u_0 and
tensor coefficients of the linear part, e.g. a viscosity nu).

The reference differentiates its integrate loop with torch autograd
(operator/_base.py:731-735 under autograd). Here the forward pass runs in
the fused CUDA kernels without a graph; the backward pass is the exact
discrete adjoint of the SETDRK4 step (integrator/_stable_etdrk/_setdrk_step.py:55-82)
written out by hand, with the forward states recomputed from checkpoints
(every ``checkpoint`` steps) segment by segment, so memory does not grow
with the step count.

Conventions. Spectral states are half spectra (last axis 0..n/2); every
cotangent is the half of a Hermitian full-spectrum cotangent v, defined by
dLoss = Re sum_k conj(v_k) du_k over the full spectrum. With F the
unnormalised DFT and N_tot the number of grid points:
  physical x -> half rfft(x)      adjoint  v -> N_tot * irfft(v)
  half a -> irfft(m a)            adjoint  x -> (m / N_tot) * rfft(x)
  half a -> irfft(i k m a)        adjoint  x -> -i k (m / N_tot) * rfft(x)
The Convection term N_c(a) = coef * rfft(sum_i u_i d_i u_c) (operator/generic/_convection.py:43-46)
has the vector-Jacobian product
  w_c = coef * N_tot * irfft(nbar_c)
  abar_c = (m / N_tot) * ( rfft(sum_c' w_c' d_c u_c') - i sum_i k_i rfft(u_i w_c) ).
Diagonal coefficients are real for the symmetric symbols this supports, so
their adjoint is the same multiplication; the coefficient cotangents are
accumulated per mode and contracted with dTable/dL * dL/dcoef, where the
table derivatives come from the FP64 contour formulas (central differences
in FP64).

One adjoint step is one call of the library's fsm_step_adjoint (the four
stages recomputed with the plan's own tables and the library's transforms,
the four vector-Jacobian products above, the backward recurrence and the
table cotangents, about 50 launches); it is captured as a CUDA graph and
replayed for every step. ``nonlinear`` / ``nonlinear_vjp`` state the same
operations with tensor arithmetic for checking.
"""

from __future__ import annotations

import ctypes
import math

import torch

from . import _lib, _native
from .integrator._standalone import RK_TABLES as _RK_TABLES


def _contour_tables(L: torch.Tensor, dt: float, M: int = 16, r: float = 1.0):
    """E, E2, c1, c4, c5, c6 of SETDRK4 for a complex128 symbol L (FP64 on L's device)."""
    j = torch.arange(1, M + 1, device=L.device, dtype=torch.float64)
    roots = torch.exp(2j * math.pi * (j - 0.5) / M)
    z = r * roots + (L * dt).unsqueeze(-1)
    ez = torch.exp(z)
    E = torch.exp(dt * L)
    E2 = torch.exp(0.5 * dt * L)
    c1 = dt * ((torch.exp(z / 2) - 1) / z).mean(-1).real
    c4 = dt * ((-4 - z + ez * (4 - 3 * z + z ** 2)) / z ** 3).mean(-1).real
    c5 = dt * ((2 + z + ez * (-2 + z)) / z ** 3).mean(-1).real
    c6 = dt * ((-4 - 3 * z - z ** 2 + ez * (4 - z)) / z ** 3).mean(-1).real
    return [E.real, E2.real, c1, c4, c5, c6]


def _table_derivatives(L: torch.Tensor, dt: float, M: int, r: float):
    """d(table)/dL for the six SETDRK4 tables of a real symbol L, in FP64: the derivatives of the same
    contour means (z = r e^{i pi (2j-1)/M} + dt L, so dz/dL = dt), term by term. E' = dt E and
    E2' = dt E2 / 2; a table c = dt mean(g(z)).real has c' = dt^2 mean(g'(z)).real, with
    g1 = (e^{z/2} - 1)/z, g1' = (z e^{z/2} / 2 - (e^{z/2} - 1))/z^2, and for the tables of the form
    g = N/z^3 (c4, c5, c6), g' = (N' z - 3 N)/z^4."""
    Lr = L.real.to(torch.complex128)
    j = torch.arange(1, M + 1, device=L.device, dtype=torch.float64)
    roots = torch.exp(2j * math.pi * (j - 0.5) / M)
    z = r * roots + (Lr * dt).unsqueeze(-1)
    ez = torch.exp(z)
    eh = torch.exp(z / 2)
    g1p = (0.5 * eh * z - (eh - 1)) / z ** 2
    n4, n4p = -4 - z + ez * (4 - 3 * z + z ** 2), -1 + ez * (1 - z + z ** 2)
    n5, n5p = 2 + z + ez * (z - 2), 1 + ez * (z - 1)
    n6, n6p = -4 - 3 * z - z ** 2 + ez * (4 - z), -3 - 2 * z + ez * (3 - z)

    def cubic(n, npr):
        return dt * dt * ((npr * z - 3 * n) / z ** 4).mean(-1).real

    return [dt * torch.exp(dt * Lr).real, 0.5 * dt * torch.exp(0.5 * dt * Lr).real, dt * dt * g1p.mean(-1).real,
            cubic(n4, n4p), cubic(n5, n5p), cubic(n6, n6p)]


class ConvectionAdjoint:
    """Forward stages and their adjoint for a Convection program (C = ndim) with a real,
    symmetric linear symbol, on one registered plan."""

    def __init__(self, plan: _native.NativePlan, program: _native.SpectralProgram, L64_half: torch.Tensor,
                 dt: float, M: int = 16, r: float = 1.0):
        if program.nonlinear != _lib.FSM_NL_CONVECTION or program.sources:
            raise NotImplementedError("the adjoint covers Convection programs without sources")
        if L64_half.is_complex() and float(L64_half.imag.abs().max()) > 0:
            raise NotImplementedError("the adjoint covers real (symmetric) linear symbols")
        self.plan = plan
        self.sp = _native.Spectral(plan)
        self.coef = float(program.nonlinear_coef)
        self.dt = float(dt)
        dev = plan.device
        shape = program.shape
        nd = len(shape)
        self.nd = nd
        self.ntot = float(math.prod(shape))
        h = shape[-1] // 2 + 1
        # wavenumbers 2 pi f on the half-spectrum grid, broadcast [1, 1, ...]
        ks = []
        for i, (s0, e0, n) in enumerate(program.mesh_info):
            idx = torch.arange(n, dtype=torch.float64, device=dev)
            idx = torch.where(idx < (n + 1) // 2, idx, idx - n)
            k = 2 * math.pi * idx / (e0 - s0)
            if i == nd - 1:
                k = k[:h]
            view = [1, 1] + [1] * nd
            view[2 + i] = k.numel()
            ks.append(k.reshape(view).to(torch.float32))
        self.k = ks
        m = torch.ones([1, 1] + [1] * nd, device=dev)
        for i in range(nd):
            keep = program.keep[i].to(dev).to(torch.float32)
            if i == nd - 1:
                keep = keep[:h]
            view = [1, 1] + [1] * nd
            view[2 + i] = keep.numel()
            m = m * keep.reshape(view)
        self.mask = m
        # mode weights of the half spectrum in full-spectrum sums (self-conjugate last-axis columns count once)
        w = torch.full((h,), 2.0, device=dev, dtype=torch.float64)
        w[0] = 1.0
        if shape[-1] % 2 == 0:
            w[-1] = 1.0
        self.weight = w
        L = L64_half.real.to(dev, torch.float64)
        self._L, self._M, self._r = L, M, r
        self._tabs = None
        self.dtabs = _table_derivatives(L.to(torch.complex128), dt, M, r)
        # dense per-point wavenumbers and mask / N_tot over the half spectrum, for the fused
        # vector-Jacobian-product combination
        half = [1, 1] + [n for n in shape[:-1]] + [h]
        self.k_dense = [torch.broadcast_to(k, half).reshape(-1).contiguous() for k in ks]
        self.m_dense = torch.broadcast_to(m / self.ntot, half).reshape(-1).contiguous().to(torch.float32)
        self.points = int(math.prod(shape))
        self.half_points = int(math.prod(shape[:-1])) * h
        self._ws = {}

    @property
    def tabs(self):
        """E, E2, c1, c4, c5, c6 from the FP64 contour formulas, rounded to FP32 (for the tensor
        formulation; the library's step reads the plan's own tables)."""
        if self._tabs is None:
            tabs = _contour_tables(self._L.to(torch.complex128), self.dt, self._M, self._r)
            self._tabs = [t.to(torch.float32) for t in tabs]
        return self._tabs

    # -- transforms --------------------------------------------------------
    def _phys(self, half):
        return self.sp.to_physical(half)

    def _spec(self, x):
        return self.sp.to_half(x)

    def _ik(self, i, x):
        return x * (1j * self.k[i])

    # -- nonlinear term and its adjoint ------------------------------------
    def _fields(self, a):
        d = a * self.mask
        u = self._phys(d)                                     # [B, C, ...]
        g = [self._phys(self._ik(i, d)) for i in range(self.nd)]  # g[i][:, c] = d_i u_c
        return u, g

    def nonlinear(self, a, keep=None):
        u, g = self._fields(a)
        if keep is not None:
            keep.append((u, g))
        p = sum(u[:, i:i + 1] * g[i] for i in range(self.nd))   # p_c = sum_i u_i d_i u_c
        return self.coef * self._spec(p)

    def nonlinear_vjp(self, a, nbar, fields=None):
        u, g = fields if fields is not None else self._fields(a)
        lib = _lib.load()
        stream = torch.cuda.current_stream(nbar.device).cuda_stream
        nb = self._phys(nbar)                                  # [B, C, ...]; w = coef N_tot nb
        B, C = nb.shape[0], nb.shape[1]
        # ubar_c = sum_c' w_c' d_c u_c' and u_i w_c in one pass over the grid
        ubar = torch.empty_like(nb)
        uw = torch.empty((self.nd,) + tuple(nb.shape), dtype=nb.dtype, device=nb.device)
        gp = [x.data_ptr() for x in g] + [None] * (3 - self.nd)
        _lib.check(lib.fsm_adj_vjp_products(B, self.nd, self.points, self.coef * self.ntot, nb.data_ptr(),
                                            u.data_ptr(), gp[0], gp[1], gp[2], ubar.data_ptr(), uw.data_ptr(),
                                            stream))
        s_ubar = self._spec(ubar)
        s_uw = self._spec(uw.reshape((self.nd * B,) + tuple(nb.shape[1:])))
        # (mask / N_tot) (rfft(ubar) - i sum_i k_i rfft(u_i w))
        out = torch.empty_like(s_ubar)
        kp = [x.data_ptr() for x in self.k_dense] + [None] * (3 - self.nd)
        _lib.check(lib.fsm_adj_vjp_combine(B * C, self.nd, self.half_points, s_ubar.data_ptr(), s_uw.data_ptr(),
                                           kp[0], kp[1], kp[2], self.m_dense.data_ptr(), out.data_ptr(), stream))
        return out

    # -- one SETDRK4 step and its adjoint --------------------------------------
    def _workspace(self, batch: int) -> torch.Tensor:
        ws = self._ws.get(batch)
        if ws is None:
            n = ctypes.c_size_t()
            _lib.check(_lib.load().fsm_step_adjoint_workspace_bytes(self.plan.handle, batch, ctypes.byref(n)))
            ws = torch.empty(int(n.value), dtype=torch.uint8, device=self.plan.device)
            self._ws[batch] = ws
        return ws

    def step_adjoint(self, u, ubar_next, tbar):
        """Cotangent of the state at the start of a step from the cotangent after it; adds the
        coefficient-table cotangents to ``tbar`` ([6, B, C, ...] float64) when given. One call of the
        library's fsm_step_adjoint (the stages recomputed with the plan's own tables)."""
        u = u.contiguous()
        ubar_next = ubar_next.contiguous()
        out = torch.empty_like(ubar_next)
        ws = self._workspace(u.shape[0])
        _lib.check(_lib.load().fsm_step_adjoint(
            self.plan.handle, u.shape[0], u.data_ptr(), ubar_next.data_ptr(), out.data_ptr(),
            tbar.data_ptr() if tbar is not None else None, ws.data_ptr(), ws.numel(),
            torch.cuda.current_stream(u.device).cuda_stream))
        return out

    def coef_gradient(self, tbar, symbol_half: torch.Tensor) -> torch.Tensor:
        """Sum over channels and modes (full spectrum) of tbar * dTable/dL * dL/dcoef, per batch entry."""
        total = 0
        for t in range(6):
            total = total + tbar[t] * self.dtabs[t]
        total = total * symbol_half.real.double() * self.weight
        return total.reshape(total.shape[0], -1).sum(-1)


class _StepGraph:
    """One adjoint step (``ConvectionAdjoint.step_adjoint``: recomputed stages, vector-Jacobian
    products, coefficient accumulation into ``tbar``) captured once as a CUDA graph and replayed
    for every step; the step is a few hundred small launches, so the replay removes their host cost.
    Inputs are copied into the graph's static buffers; the returned cotangent is the graph's
    static output, valid until the next call."""

    def __init__(self, adj: "ConvectionAdjoint", like: torch.Tensor, tbar):
        dev = like.device
        self.u_in = torch.zeros_like(like)
        self.v_in = torch.zeros_like(like)
        scratch = torch.zeros_like(tbar) if tbar is not None else None
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            adj.step_adjoint(self.u_in, self.v_in, scratch)  # warm-up: kernel attributes, allocator
        torch.cuda.current_stream(dev).wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.v_out = adj.step_adjoint(self.u_in, self.v_in, tbar)

    def __call__(self, u: torch.Tensor, v: torch.Tensor) -> torch.Tensor:
        self.u_in.copy_(u)
        self.v_in.copy_(v)
        self.graph.replay()
        return self.v_out


class _IntegrateFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, adj, steps, checkpoint, symbols, *coefs):
        plan = adj.plan
        sp = adj.sp
        state = sp.to_half(u0.detach()).contiguous()
        checkpoints = [state.clone()]
        done = 0
        while done < steps:
            k = min(checkpoint, steps - done)
            plan.integrate_half(state, k)
            done += k
            if done < steps:
                checkpoints.append(state.clone())
        ctx.adj, ctx.steps, ctx.checkpoint, ctx.symbols = adj, steps, checkpoint, symbols
        ctx.checkpoints = checkpoints
        ctx.n_coefs = len(coefs)
        ctx.coef_shapes = [c.shape for c in coefs]
        return sp.to_physical(state, keep_input=False)

    @staticmethod
    def backward(ctx, grad_out):
        adj = ctx.adj
        plan = adj.plan
        steps, K = ctx.steps, ctx.checkpoint
        v = adj._spec(grad_out.contiguous().float()) / adj.ntot
        want_coef = any(ctx.needs_input_grad[5:])
        tbar = None
        if want_coef:
            tbar = torch.zeros((6,) + tuple(v.shape), dtype=torch.float64, device=v.device)
        step = _StepGraph(adj, v, tbar) if steps > 1 else None
        starts = list(range(0, steps, K))
        for si in reversed(range(len(starts))):
            start = starts[si]
            n = min(K, steps - start)
            # recompute the segment's states with the fused kernel (one recorded frame per step)
            st = ctx.checkpoints[si].clone()
            frames = torch.empty((st.shape[0], n) + tuple(st.shape[1:]), dtype=torch.complex64, device=st.device)
            plan.integrate_half(st, n - 1, slots=list(range(n)), traj=frames) if n > 1 else frames[:, 0].copy_(st)
            for j in reversed(range(n)):
                if step is not None:
                    v = step(frames[:, j], v)
                else:
                    v = adj.step_adjoint(frames[:, j].contiguous(), v, tbar)
        v = v.clone()
        grad_u0 = adj.ntot * adj.sp.to_physical(v) if ctx.needs_input_grad[0] else None
        grads = [None] * ctx.n_coefs
        if want_coef:
            for i, (sym, shp) in enumerate(zip(ctx.symbols, ctx.coef_shapes)):
                if not ctx.needs_input_grad[5 + i]:
                    continue
                per_batch = adj.coef_gradient(tbar, sym)
                g = per_batch if len(shp) > 0 and shp.numel() > 1 else per_batch.sum()
                grads[i] = g.reshape(shp).to(torch.float32) if len(shp) > 0 else g.to(torch.float32)
        return (grad_u0, None, None, None, None, *grads)


def _scheme_tables(scheme: int, L: torch.Tensor, dt: float, M: int, r: float) -> dict:
    """The coefficient tables of an integration scheme as torch functions of the complex128 symbol L,
    which autograd differentiates with respect to L (and so to the coefficients in L).

    SETDRK1-4: the means over M contour points z = r e^{i pi (2j-1)/M} + dt L of the reference's
    integrands, real parts kept (integrator/_stable_etdrk/_uncached.py:8-43, 46-211); ETDRK0-2: the
    closed forms with their L == 0 limits, complex (integrator/_etdrk.py:10-82; the limits are
    selected without the 0/0 of the other branch, so their gradients stay finite); Runge-Kutta: the
    symbol itself (the slopes are dt (L x + N(x)), operator/_base.py:408-431)."""
    if scheme in _RK_TABLES:
        return {"L": L}
    E = torch.exp(dt * L)
    if scheme in (_lib.FSM_ETDRK0, _lib.FSM_ETDRK1, _lib.FSM_ETDRK2):
        out = {"E": E}
        zero = L == 0
        Ls = torch.where(zero, torch.ones_like(L), L)
        if scheme != _lib.FSM_ETDRK0:
            out["c1"] = torch.where(zero, torch.full_like(L, dt), (E - 1) / Ls)
        if scheme == _lib.FSM_ETDRK2:
            out["c2"] = torch.where(zero, torch.full_like(L, dt / 2), (E - 1 - Ls * dt) / (Ls ** 2 * dt))
        return out
    j = torch.arange(1, M + 1, device=L.device, dtype=torch.float64)
    roots = torch.exp(2j * math.pi * (j - 0.5) / M)
    z = r * roots + (L * dt).unsqueeze(-1)
    ez = torch.exp(z)

    def mean(expr):
        return dt * expr.mean(-1).real

    out = {"E": E}
    if scheme in (_lib.FSM_SETDRK1, _lib.FSM_SETDRK2):
        out["c1"] = mean((ez - 1) / z)
        if scheme == _lib.FSM_SETDRK2:
            out["c2"] = mean((ez - 1 - z) / z ** 2)
    elif scheme == _lib.FSM_SETDRK3:
        out["E2"] = torch.exp(0.5 * dt * L)
        out["c1"] = mean((torch.exp(z / 2) - 1) / z)
        out["c2"] = mean((ez - 1) / z)
        out["c3"] = mean((-4 - z + ez * (4 - 3 * z + z ** 2)) / z ** 3)
        out["c4"] = mean((4.0 * (2.0 + z + ez * (-2 + z))) / z ** 3)
        out["c5"] = mean((-4 - 3 * z - z ** 2 + ez * (4 - z)) / z ** 3)
    elif scheme == _lib.FSM_SETDRK4:
        out["E2"] = torch.exp(0.5 * dt * L)
        out["c1"] = mean((torch.exp(z / 2) - 1) / z)
        out["c4"] = mean((-4 - z + ez * (4 - 3 * z + z ** 2)) / z ** 3)
        out["c5"] = mean((2 + z + ez * (-2 + z)) / z ** 3)
        out["c6"] = mean((-4 - 3 * z - z ** 2 + ez * (4 - z)) / z ** 3)
    else:
        raise NotImplementedError(f"gradients: integrator code {scheme}")
    return out


def _scheme_step(scheme: int, u: torch.Tensor, T: dict, nonlinear, dt: float) -> torch.Tensor:
    """One step of the scheme on full spectra in torch arithmetic: the stage recurrences of
    integrator/_etdrk.py:22-82 (ETDRK0-2), _stable_etdrk/_setdrk_step.py:5-82 (SETDRK1-4) and the
    fixed Runge-Kutta step of integrator/_rk.py:43-58 with its tableau."""
    if scheme in _RK_TABLES:
        L = T["L"]

        def rhs(x):
            return L * x if nonlinear is None else L * x + nonlinear(x)

        rows, weights = _RK_TABLES[scheme]
        ks = [rhs(u)]
        for row in rows:
            ks.append(rhs(u + dt * sum(a * k for a, k in zip(row[1:], ks))))
        return u + dt * sum(w * k for w, k in zip(weights, ks))
    E = T["E"]
    if scheme == _lib.FSM_ETDRK0:
        return E * u
    if scheme in (_lib.FSM_ETDRK1, _lib.FSM_SETDRK1):
        return E * u + T["c1"] * nonlinear(u)
    if scheme in (_lib.FSM_ETDRK2, _lib.FSM_SETDRK2):
        n0 = nonlinear(u)
        a1 = E * u + T["c1"] * n0
        return a1 + T["c2"] * (nonlinear(a1) - n0)
    E2, c1 = T["E2"], T["c1"]
    n0 = nonlinear(u)
    a1 = E2 * u + c1 * n0
    n1 = nonlinear(a1)
    if scheme == _lib.FSM_SETDRK3:
        a2 = E * u + T["c2"] * (2 * n1 - n0)
        n2 = nonlinear(a2)
        return E * u + T["c3"] * n0 + T["c4"] * n1 + T["c5"] * n2
    a2 = E2 * u + c1 * n1
    n2 = nonlinear(a2)
    a3 = E2 * a1 + c1 * (2 * n2 - n0)
    n3 = nonlinear(a3)
    return E * u + T["c4"] * n0 + T["c5"] * 2 * (n1 + n2) + T["c6"] * n3


class _RecomputeFn(torch.autograd.Function):
    """Gradients of an integration of any program (vorticity, KS, Leray, sources, complex symbols,
    Python-callable terms) under any fixed-step scheme (ETDRK0-2, SETDRK1-4, the Runge-Kutta
    schemes): the forward runs the library's integration with checkpoints every ``checkpoint``
    steps; the backward recomputes each segment from its checkpoint with the same step written in
    torch arithmetic on full spectra (the operator's own nonlinear closure, the scheme's tables from
    the FP64 formulas of the operator's linear symbol, rounded to FP32) and differentiates that
    segment with torch autograd, last segment first. Only one segment's graph is alive at a time."""

    @staticmethod
    def forward(ctx, u0, op, plan, spectral, dt, steps, checkpoint, scheme, *coefs):
        state = spectral.to_half(u0.detach()).contiguous()
        checkpoints = [state.clone()]
        done = 0
        while done < steps:
            k = min(checkpoint, steps - done)
            plan.integrate_half(state, k)
            done += k
            if done < steps:
                checkpoints.append(state.clone())
        ctx.op, ctx.spectral, ctx.dt, ctx.steps, ctx.checkpoint = op, spectral, dt, steps, checkpoint
        ctx.scheme = scheme
        ctx.checkpoints = checkpoints
        ctx.save_for_backward(u0, *coefs)
        return spectral.to_physical(state, keep_input=False)

    @staticmethod
    def backward(ctx, grad_out):
        op, sp = ctx.op, ctx.spectral
        u0, *coefs = ctx.saved_tensors
        steps, K, dt = ctx.steps, ctx.checkpoint, ctx.dt
        f_mesh = op._state_dict["f_mesh"]
        C = op._state_dict["n_channel"]
        nd = len(f_mesh.mesh_info)
        dims = tuple(range(-nd, 0))
        from .mesh import FourierMesh

        fm64 = FourierMesh(f_mesh.mesh_info, device=u0.device, dtype=torch.float64)
        cfg = getattr(op, "_integrator_config", {}) or {}
        M = int(cfg.get("n_integration_points", 16))
        r = float(cfg.get("integration_radius", 1.0))
        nonlinear = op._state_dict["nonlinear_func"]
        with torch.enable_grad():
            leaves = [c.detach().requires_grad_(ctx.needs_input_grad[8 + i]) for i, c in enumerate(coefs)]
            by_id = {id(c): leaf for c, leaf in zip(coefs, leaves)}
            L = None
            for coef, core in op._linear_terms:
                if isinstance(coef, torch.Tensor):
                    c64 = by_id.get(id(coef), coef.detach()).to(device=u0.device, dtype=torch.float64)
                else:
                    c64 = coef
                term = c64 * core(fm64, C)
                L = term if L is None else L + term
            if L is None:
                L = torch.zeros((1, 1) + (1,) * nd, dtype=torch.complex128, device=u0.device)
            tabs = {k: (t.to(torch.complex64) if t.is_complex() else t.to(torch.float32))
                    for k, t in _scheme_tables(ctx.scheme, L.to(torch.complex128), dt, M, r).items()}
            v = grad_out.to(torch.float32)
            coef_grads = [None] * len(coefs)
            starts = list(range(0, steps, K))
            u0_grad = None
            for si in reversed(range(len(starts))):
                n = min(K, steps - starts[si])
                if si == 0:
                    x_in = u0.detach().to(torch.float32).requires_grad_(ctx.needs_input_grad[0])
                    y = torch.fft.fftn(x_in, dim=dims).to(torch.complex64)
                else:
                    x_in = sp.half_to_full(ctx.checkpoints[si]).to(torch.complex64).detach().requires_grad_(True)
                    y = x_in
                for _ in range(n):
                    y = _scheme_step(ctx.scheme, y, tabs, nonlinear, dt)
                out = torch.fft.ifftn(y, dim=dims).real if si == len(starts) - 1 else y
                wanted = [x_in] + [leaf for leaf in leaves if leaf.requires_grad]
                grads = torch.autograd.grad(out, wanted, grad_outputs=v, allow_unused=True,
                                            retain_graph=si > 0)
                j = 1
                for i, leaf in enumerate(leaves):
                    if leaf.requires_grad:
                        g = grads[j]
                        j += 1
                        if g is not None:
                            coef_grads[i] = g if coef_grads[i] is None else coef_grads[i] + g
                if si == 0:
                    u0_grad = grads[0]
                else:
                    v = grads[0].detach()
        grads_out = [u0_grad.to(u0.dtype) if (u0_grad is not None and ctx.needs_input_grad[0]) else None]
        grads_out += [None] * 7
        for i, c in enumerate(coefs):
            g = coef_grads[i]
            grads_out.append(g.to(c.dtype).reshape(c.shape) if g is not None else None)
        return tuple(grads_out)


def integrate_with_grad(op, u0: torch.Tensor, dt: float, steps: int, checkpoint: int = 50) -> torch.Tensor:
    """``op.integrate(u_0=u0, dt=dt, step=steps)`` with gradients to u0 and to tensor coefficients
    of the operator's linear terms (the operator's mesh must be registered)."""
    with torch.no_grad():
        return _prepare_and_apply(op, u0, dt, steps, checkpoint)


def _convection_adjoint_applies(op, plan) -> bool:
    """The hand-written adjoint's programs: fused Convection (C == ndim) without sources, with a real
    linear symbol."""
    if not isinstance(plan, _native.NativePlan):
        return False
    prog = plan.program
    if prog.nonlinear != _lib.FSM_NL_CONVECTION or prog.sources:
        return False
    L64 = op._linear_coef64(plan.device)
    return not (L64.is_complex() and float(L64.imag.abs().max()) > 0)


def _prepare_and_apply(op, u0, dt, steps, checkpoint):
    integ = op._state_dict["integrator"]
    if integ is None or integ.dt != dt or integ.plan.device != u0.device:
        op._build_integrator(dt, u0.device)
        integ = op._state_dict["integrator"]
    plan = integ.plan
    scheme = int(plan.integrator)
    coefs = [c for c, _ in op._linear_terms if isinstance(c, torch.Tensor) and c.requires_grad]
    if scheme != _lib.FSM_SETDRK4 or not _convection_adjoint_applies(op, plan):
        # any other program or scheme: segments recomputed and differentiated with torch autograd
        with torch.enable_grad():
            return _RecomputeFn.apply(u0, op, plan, integ.spectral, float(dt), int(steps), int(checkpoint), scheme,
                                      *coefs)
    prog = plan.program
    L64 = op._linear_coef64(u0.device)
    h = plan.shape[-1] // 2 + 1
    nd = len(plan.shape)
    L64 = L64.expand(L64.shape[:2] + tuple(plan.shape))[..., :h]
    adj = ConvectionAdjoint(plan, prog, L64, dt)
    coefs, symbols = [], []
    C = op._state_dict["n_channel"]
    f_mesh = op._state_dict["f_mesh"]
    from .mesh import FourierMesh

    fm64 = FourierMesh(f_mesh.mesh_info, device=u0.device, dtype=torch.float64)
    for coef, core in op._linear_terms:
        if isinstance(coef, torch.Tensor) and coef.requires_grad:
            sym = core(fm64, C)
            sym = sym.expand(sym.shape[:2] + tuple(plan.shape))[..., :h].contiguous()
            coefs.append(coef)
            symbols.append(sym)
    with torch.enable_grad():
        return _IntegrateFn.apply(u0, adj, int(steps), int(checkpoint), symbols, *coefs)
