"""numpy restatement of torchfsm's Fourier-spectral ETD path (the oracle).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``). Full complex C2C
spectra as in the reference; FP64 by default. ``real_dtype=np.float32`` runs
the same algorithm in complex64 and is used only as the timed CPU restatement
of the reference's FP32 run in ``bench.py``.

Every function cites the reference (torchfsm 0.0.4) file:line it restates.
"""

from __future__ import annotations

import math
from typing import Callable, List, Optional, Sequence, Tuple

import numpy as np

# ----------------------------------------------------------------------------
# mesh: torchfsm/mesh.py
# ----------------------------------------------------------------------------


def fftfreq(n: int, length: float, real_dtype=np.float64) -> np.ndarray:
    """Cycles per unit length, ``torch.fft.fftfreq(n, length/n)`` (mesh.py:185-191)."""
    return np.fft.fftfreq(n, d=length / n).astype(real_dtype)


class OMesh:
    """FourierMesh restated (mesh.py:294-505) on a list of (start, end, n).

    ``bf[i]`` is the broadcast frequency of axis i with shape
    ``[1, 1, 1.., N_i, ..1]`` (mesh.py:244-254).
    """

    def __init__(self, mesh_info: Sequence[Tuple[float, float, int]], real_dtype=np.float64):
        self.mesh_info = [tuple(m) for m in mesh_info]
        self.n_dim = len(self.mesh_info)
        self.real_dtype = np.dtype(real_dtype)
        self.complex_dtype = np.result_type(self.real_dtype, np.complex64)
        self.shape = tuple(int(m[2]) for m in self.mesh_info)
        self.fft_axes = tuple(-(i + 1) for i in range(self.n_dim))
        self.bf = []
        for i, (s, e, n) in enumerate(self.mesh_info):
            f = fftfreq(int(n), e - s, self.real_dtype)
            shape = [1] * (self.n_dim + 2)
            shape[i + 2] = int(n)
            self.bf.append(f.reshape(shape))

    # mesh.py:399-404
    def grad(self, dim_i: int, order: int) -> np.ndarray:
        return ((2j * math.pi * self.bf[dim_i]) ** order).astype(self.complex_dtype)

    # mesh.py:421-426
    def nabla(self, order: int = 1) -> np.ndarray:
        out = 0
        for i in range(self.n_dim):
            out = out + self.grad(i, order)
        return np.broadcast_to(out, (1, 1) + self.shape).astype(self.complex_dtype)

    # mesh.py:406-411
    def laplacian(self) -> np.ndarray:
        return self.nabla(2)

    # mesh.py:413-419: 1/lap with 1.0 where lap == 0
    def invert_laplacian(self) -> np.ndarray:
        lap = self.laplacian()
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = np.where(lap == 0, 1.0, 1.0 / np.where(lap == 0, 1.0, lap))
        return inv.astype(self.complex_dtype)

    # mesh.py:436-441: [1, d, N..]
    def nabla_vector(self, order: int = 1) -> np.ndarray:
        comps = [np.broadcast_to(self.grad(i, order), (1, 1) + self.shape) for i in range(self.n_dim)]
        return np.concatenate(comps, axis=1)

    # mesh.py:443-461: product over axes of [|f_i| <= rate * max|f_i|]
    def low_pass_filter(self, rate: float = 2.0 / 3.0) -> np.ndarray:
        mask = np.ones((1, 1) + self.shape, dtype=self.real_dtype)
        for i in range(self.n_dim):
            a = np.abs(self.bf[i])
            thr = self.real_dtype.type(a.max() * self.real_dtype.type(rate))
            mask = mask * np.where(a > thr, 0, 1).astype(self.real_dtype)
        return mask

    # mesh.py:481-491 ("backward" normalisation: 1/N on the inverse)
    def fft(self, u: np.ndarray) -> np.ndarray:
        return np.fft.fftn(u, axes=self.fft_axes).astype(self.complex_dtype, copy=False)

    def ifft(self, u_fft: np.ndarray) -> np.ndarray:
        return np.fft.ifftn(u_fft, axes=self.fft_axes).astype(self.complex_dtype, copy=False)


# ----------------------------------------------------------------------------
# linear cores: operator/generic/_laplacian.py, _biharmonic.py,
# _spatial_derivative.py, _source.py
# ----------------------------------------------------------------------------


def linear_symbol(mesh: OMesh, terms: Sequence[Tuple[object, tuple]], n_channel: int) -> np.ndarray:
    """Sum of coef * symbol (operator/_base.py:339-357).

    ``terms`` holds (coef, spec) with spec one of ("laplacian",),
    ("biharmonic",), ("spatial_derivative", dim, order), ("unit",).
    ``coef`` may be a scalar or an array broadcastable to [B, 1, 1..].
    """
    total = 0
    for coef, spec in terms:
        kind = spec[0]
        if kind == "laplacian":  # _laplacian.py:7-15 (cat over channels)
            sym = np.concatenate([mesh.laplacian()] * n_channel, axis=1)
        elif kind == "biharmonic":  # _biharmonic.py:8-16
            lap = mesh.laplacian()
            sym = np.concatenate([lap * lap] * n_channel, axis=1)
        elif kind == "spatial_derivative":  # _spatial_derivative.py:7-20
            sym = mesh.grad(spec[1], spec[2])
        elif kind == "unit":  # _source.py:9-17
            sym = np.ones_like(mesh.bf[0]).astype(mesh.complex_dtype)
        else:
            raise ValueError(kind)
        total = total + np.asarray(coef) * sym
    return np.asarray(total).astype(mesh.complex_dtype)


# ----------------------------------------------------------------------------
# nonlinear cores
# ----------------------------------------------------------------------------


def convection(u_fft, mesh: OMesh, u=None):
    """(u.grad)u, operator/generic/_convection.py:18-46."""
    if u is None:
        u = mesh.ifft(u_fft).real
    nabla_u = mesh.nabla_vector(1)[:, :, None] * u_fft[:, None]  # [B, d, C, ..]
    phys = (u[:, :, None] * mesh.ifft(nabla_u).real).sum(1)
    return mesh.fft(phys)


def vorticity_convection(u_fft, mesh: OMesh, u=None):
    """u.grad(omega) via the streamfunction, operator/dedicated/_navier_stokes.py:27-46."""
    psi = -u_fft * mesh.invert_laplacian()
    ux = mesh.ifft(mesh.grad(1, 1) * psi).real
    uy = mesh.ifft(-mesh.grad(0, 1) * psi).real
    wx = mesh.ifft(mesh.grad(0, 1) * u_fft).real
    wy = mesh.ifft(mesh.grad(1, 1) * u_fft).real
    return mesh.fft(ux * wx + uy * wy)


def ks_convection(u_fft, mesh: OMesh, u=None, remove_mean: bool = True):
    """0.5|grad phi|^2, operator/dedicated/_ks_convection.py:18-38.

    The mean removed is ``re.mean()`` over the WHOLE tensor, batch included
    (_ks_convection.py:35-36).
    """
    grad_u = mesh.ifft(mesh.nabla_vector(1) * u_fft).real
    re = 0.5 * np.sum(grad_u ** 2, axis=1, keepdims=True)
    if remove_mean:
        re = re - re.mean()
    return mesh.fft(re)


def conservative_convection(u_fft, mesh: OMesh, u=None):
    """div(uu), operator/generic/_conservative_convection.py:18-27."""
    if u is None:
        u = mesh.ifft(u_fft).real
    uu = u[:, :, None] * u[:, None]
    uu_fft = mesh.fft(uu)
    return (mesh.nabla_vector(1)[:, :, None] * uu_fft).sum(1)


def ns_pressure_convection(u_fft, mesh: OMesh, u=None):
    """-grad p - (u.grad)u (Leray projection), operator/dedicated/_navier_stokes.py:231-254
    without external force."""
    if u is None:
        u = mesh.ifft(u_fft).real
    conv = convection(u_fft, mesh, u)
    nv = mesh.nabla_vector(1)
    p = mesh.invert_laplacian() * np.sum(nv * conv, axis=1, keepdims=True)
    return nv * p - conv


NONLINEAR = {
    "convection": (convection, True),
    "vorticity_convection": (vorticity_convection, True),
    "ks_convection": (lambda uf, m, u=None: ks_convection(uf, m, u, True), True),
    "ks_convection_keep_mean": (lambda uf, m, u=None: ks_convection(uf, m, u, False), True),
    "conservative_convection": (conservative_convection, True),
    "ns_pressure_convection": (ns_pressure_convection, True),
}


def make_nonlinear(mesh: OMesh, terms: Sequence[Tuple[object, object]], de_aliasing_rate: float = 2.0 / 3.0):
    """Dealiased sum of nonlinear cores, operator/_base.py:359-406.

    ``terms``: (coef, name) with name a key of NONLINEAR, or (coef, ("source", S_fft))
    for an explicit source (operator/_base.py:994-1015, no dealiasing).
    The input (not the output) is masked.
    """
    if len(terms) == 0:
        return None
    mask = mesh.low_pass_filter(de_aliasing_rate)

    def nonlinear_all(u_fft):
        result = 0.0
        d_fft = None
        d_u = None
        for coef, name in terms:
            if isinstance(name, tuple) and name[0] == "source":
                result = result + coef * name[1]
                continue
            fun, dealias = NONLINEAR[name]
            if dealias:
                if d_fft is None:
                    d_fft = u_fft * mask
                    d_u = mesh.ifft(d_fft).real
                result = result + coef * fun(d_fft, mesh, d_u)
            else:
                result = result + coef * fun(u_fft, mesh, None)
        return result

    return nonlinear_all


# ----------------------------------------------------------------------------
# integrators: integrator/_etdrk.py, integrator/_stable_etdrk/
# ----------------------------------------------------------------------------


def roots_of_unity(m: int, real_dtype=np.float64) -> np.ndarray:
    """exp(2 pi i (j - 1/2)/M), j = 1..M (_stable_etdrk/_uncached.py:8-15)."""
    j = np.arange(1, m + 1, dtype=real_dtype)
    return np.exp(2j * np.pi * (j - 0.5) / m)


def contour_points(lin: np.ndarray, dt: float, m: int, r: float) -> np.ndarray:
    """lr = r * roots + L * dt on a trailing axis (_uncached.py:34-43)."""
    rd = np.real(lin).dtype
    return r * roots_of_unity(m, rd) + lin[..., None] * dt


def setdrk_coefs(order: int, lin: np.ndarray, dt: float, m: int = 16, r: float = 1.0) -> dict:
    """Coefficient tables of UnCachedSETDRK1..4 (_uncached.py:46-211)."""
    lin = np.asarray(lin)
    out = {"E": np.exp(dt * lin)}  # _uncached.py:30
    lr = contour_points(lin, dt, m, r)
    el = np.exp(lr)

    def mean_real(expr):
        return dt * np.mean(expr, axis=-1).real

    if order == 1:
        out["c1"] = mean_real((el - 1) / lr)
    elif order == 2:
        out["c1"] = mean_real((el - 1) / lr)
        out["c2"] = mean_real((el - 1 - lr) / lr ** 2)
    elif order == 3:
        out["E2"] = np.exp(0.5 * dt * lin)
        out["c1"] = mean_real((np.exp(lr / 2) - 1) / lr)
        out["c2"] = mean_real((el - 1) / lr)
        out["c3"] = mean_real((-4 - lr + el * (4 - 3 * lr + lr ** 2)) / lr ** 3)
        out["c4"] = mean_real((4.0 * (2.0 + lr + el * (-2 + lr))) / lr ** 3)
        out["c5"] = mean_real((-4 - 3 * lr - lr ** 2 + el * (4 - lr)) / lr ** 3)
    elif order == 4:
        out["E2"] = np.exp(0.5 * dt * lin)
        c1 = mean_real((np.exp(lr / 2) - 1) / lr)
        out["c1"] = out["c2"] = out["c3"] = c1
        out["c4"] = mean_real((-4 - lr + el * (4 - 3 * lr + lr ** 2)) / lr ** 3)
        out["c5"] = mean_real((2 + lr + el * (-2 + lr)) / lr ** 3)
        out["c6"] = mean_real((-4 - 3 * lr - lr ** 2 + el * (4 - lr)) / lr ** 3)
    else:
        raise ValueError(order)
    return out


def etdrk_coefs(order: int, lin: np.ndarray, dt: float) -> dict:
    """ETDRK0/1/2 coefficient tables (integrator/_etdrk.py:10-82)."""
    lin = np.asarray(lin)
    e = np.exp(dt * lin)
    out = {"E": e}
    with np.errstate(divide="ignore", invalid="ignore"):
        if order >= 1:
            out["c1"] = np.where(lin == 0, dt, (e - 1) / lin)
        if order >= 2:
            out["c2"] = np.where(lin == 0, dt / 2, (e - 1 - lin * dt) / (lin ** 2 * dt))
    return out


def stage_step(name: str, tabs: dict, nonlinear: Callable, u: np.ndarray) -> np.ndarray:
    """One step of the named scheme.

    setdrk1..4: _stable_etdrk/_setdrk_step.py:5-82; etdrk0..2: _etdrk.py:22-82.
    """
    if name in RK_TABLEAUS:
        # f(u) = L u + N(u) (operator/_base.py:408-431)
        L = tabs["L"]
        rhs = (lambda x: L * x) if nonlinear is None else (lambda x: L * x + nonlinear(x))
        return rk_step(name, rhs, u, tabs["dt"])
    E = tabs["E"]
    if name == "etdrk0":
        return E * u
    if name in ("etdrk1", "setdrk1"):
        return E * u + tabs["c1"] * nonlinear(u)
    if name == "etdrk2":
        n0 = nonlinear(u)
        a1 = E * u + tabs["c1"] * n0
        n1 = nonlinear(a1)
        return a1 + tabs["c2"] * (n1 - n0)
    if name == "setdrk2":
        n0 = nonlinear(u)
        a1 = E * u + tabs["c1"] * n0
        n1 = nonlinear(a1)
        return a1 + tabs["c2"] * (n1 - n0)
    if name == "setdrk3":
        E2 = tabs["E2"]
        n0 = nonlinear(u)
        a1 = E2 * u + tabs["c1"] * n0
        n1 = nonlinear(a1)
        a2 = E * u + tabs["c2"] * (2 * n1 - n0)
        n2 = nonlinear(a2)
        return E * u + tabs["c3"] * n0 + tabs["c4"] * n1 + tabs["c5"] * n2
    if name == "setdrk4":
        E2 = tabs["E2"]
        n0 = nonlinear(u)
        a1 = E2 * u + tabs["c1"] * n0
        n1 = nonlinear(a1)
        a2 = E2 * u + tabs["c2"] * n1
        n2 = nonlinear(a2)
        a3 = E2 * a1 + tabs["c3"] * (2 * n2 - n0)
        n3 = nonlinear(a3)
        return E * u + tabs["c4"] * n0 + tabs["c5"] * 2 * (n1 + n2) + tabs["c6"] * n3
    raise ValueError(name)


# Explicit Runge-Kutta tableaus by the reference's enum names (integrator/_rk.py:82-255):
# (rows of [c_i, a_i0, a_i1, ...] for the stages after the first, weights b).
RK_TABLEAUS = {
    "Euler": ([[1.0]], [1.0]),
    "Midpoint": ([[1 / 2, 1 / 2]], [0, 1]),
    "Heun12": ([[1, 1]], [1 / 2, 1 / 2]),
    "Ralston12": ([[2 / 3, 2 / 3]], [1 / 4, 3 / 4]),
    "BogackiShampine23": ([[1 / 2, 1 / 2], [3 / 4, 0, 3 / 4], [1, 2 / 9, 1 / 3, 4 / 9]], [2 / 9, 1 / 3, 4 / 9, 0]),
    "RK4": ([[1 / 2, 1 / 2], [1 / 2, 0, 1 / 2], [1, 0, 0, 1]], [1 / 6, 1 / 3, 1 / 3, 1 / 6]),
    # the last row, read with the first entry as c like every other row, gives a3 = (-1, 1, 1)
    # (the textbook 3/8 rule has (1, -1, 1)): the reference runs it that way, and so does this
    "RK4_38Rule": ([[1 / 3, 1 / 3], [2 / 3, -1 / 3, 1], [1, -1, 1, 1]], [1 / 8, 3 / 8, 3 / 8, 1 / 8]),
    "Dorpi45": ([[1 / 5, 1 / 5], [3 / 10, 3 / 40, 9 / 40], [4 / 5, 44 / 45, -56 / 15, 32 / 9],
                 [8 / 9, 19372 / 6561, -25360 / 2187, 64448 / 6561, -212 / 729],
                 [1, 9017 / 3168, -355 / 33, 46732 / 5247, 49 / 176, -5103 / 18656],
                 [1, 35 / 384, 0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84]],
                [35 / 384, 0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84]),
    "Fehlberg45": ([[1 / 4, 1 / 4], [3 / 8, 3 / 32, 9 / 32], [12 / 13, 1932 / 2197, -7200 / 2197, 7296 / 2197],
                    [1, 439 / 216, -8, 3680 / 513, -845 / 4104], [1 / 2, -8 / 27, 2, -3544 / 2565, 1859 / 4104, -11 / 40]],
                   [16 / 135, 0, 6656 / 12825, 28561 / 56430, -9 / 50, 2 / 55]),
    "CashKarp45": ([[1 / 5, 1 / 5], [3 / 10, 3 / 40, 9 / 40], [3 / 5, 3 / 10, -9 / 10, 6 / 5],
                    [1, -11 / 54, 5 / 2, -70 / 27, 35 / 27],
                    [7 / 8, 1631 / 55296, 175 / 512, 575 / 13824, 44275 / 110592, 253 / 4096]],
                   [37 / 378, 0, 250 / 621, 125 / 594, 0, 512 / 1771]),
}


def rk_step(name: str, rhs: Callable, x: np.ndarray, dt: float) -> np.ndarray:
    """One fixed step of an explicit Runge-Kutta scheme (integrator/_rk.py:43-58, _rk_step):
    k_0 = f(x), k_{i+1} = f(x + dt sum_j a_ij k_j), x' = x + dt sum_i b_i k_i (sums truncated to the
    slopes available, as the reference's zip does)."""
    ca, b = RK_TABLEAUS[name]
    ks = [rhs(x)]
    for row in ca:
        ks.append(rhs(x + dt * sum(a * k for a, k in zip(row[1:], ks))))
    return x + dt * sum(w * k for w, k in zip(b, ks))


def build_tables(name: str, lin: np.ndarray, dt: float, m: int = 16, r: float = 1.0) -> dict:
    if name in RK_TABLEAUS:
        return {"L": np.asarray(lin), "dt": dt}
    if name.startswith("setdrk"):
        return setdrk_coefs(int(name[-1]), lin, dt, m, r)
    return etdrk_coefs(int(name[-1]), lin, dt)


def integrate(
    u0: np.ndarray,
    mesh_info,
    linear_terms,
    nonlinear_terms,
    dt: float,
    step: int,
    integrator: str = "auto",
    record: Optional[Callable[[int], bool]] = None,
    de_aliasing_rate: float = 2.0 / 3.0,
    n_integration_points: int = 16,
    integration_radius: float = 1.0,
    real_dtype=np.float64,
    u0_fft: Optional[np.ndarray] = None,
    return_in_fourier: bool = False,
):
    """Operator.integrate restated (operator/_base.py:676-751).

    ``integrator="auto"``: ETDRK0 for linear-only programs, SETDRK4 otherwise
    (_base.py:451-455). A program without linear terms integrates with L = 0
    (_base.py:473-478). ``record(step)`` plays the recorder's control function
    (traj_recorder.py:46-55): frames are the states before each step and after
    the last one. Returns ``(final, trajectory_or_None)`` in physical space
    (real) unless ``return_in_fourier``.
    """
    mesh = OMesh(mesh_info, real_dtype)
    src = u0 if u0 is not None else u0_fft
    n_channel = src.shape[1]
    nonlinear = make_nonlinear(mesh, nonlinear_terms, de_aliasing_rate)
    if linear_terms:
        lin = linear_symbol(mesh, linear_terms, n_channel)
    else:
        lin = np.zeros((1,), dtype=mesh.complex_dtype)
    if integrator == "auto":
        integrator = "etdrk0" if nonlinear is None else "setdrk4"
    tabs = build_tables(integrator, lin, dt, n_integration_points, integration_radius)
    tabs = {k: (v if k == "dt" else np.asarray(v).astype(mesh.complex_dtype if np.iscomplexobj(v) else mesh.real_dtype))
            for k, v in tabs.items()}
    u_hat = mesh.fft(u0.astype(real_dtype)) if u0_fft is None else u0_fft.astype(mesh.complex_dtype)
    frames: List[np.ndarray] = []
    for i in range(step):
        if record is not None and record(i):
            frames.append(u_hat.copy())
        u_hat = stage_step(integrator, tabs, nonlinear, u_hat)
    if record is not None and record(step):
        frames.append(u_hat.copy())
    traj = None
    if record is not None:
        traj = np.stack(frames, axis=1) if frames else None
        if traj is not None and not return_in_fourier:
            traj = np.fft.ifftn(traj, axes=tuple(-(i + 1) for i in range(mesh.n_dim))).real
    final = u_hat if return_in_fourier else mesh.ifft(u_hat).real
    return final, traj


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """||a - b|| / ||b|| over all entries."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def apply_operator(u: np.ndarray, mesh_info, linear_terms, nonlinear_terms, de_aliasing_rate: float = 2.0 / 3.0,
                   real_dtype=np.float64) -> np.ndarray:
    """One evaluation ifft(L u_hat + N(u_hat)).real (operator/_base.py:408-431, 753-790)."""
    mesh = OMesh(mesh_info, real_dtype)
    u_hat = mesh.fft(np.asarray(u, dtype=real_dtype))
    out = np.zeros_like(u_hat)
    if linear_terms:
        out = out + linear_symbol(mesh, linear_terms, u.shape[1]) * u_hat
    nonlinear = make_nonlinear(mesh, nonlinear_terms, de_aliasing_rate)
    if nonlinear is not None:
        out = out + nonlinear(u_hat)
    return mesh.ifft(out).real
