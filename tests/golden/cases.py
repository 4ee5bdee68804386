"""Parity cases shared by the golden-vector generator, the oracle tests and the GPU tests.

Each case names: the mesh, how to build the operator from a torchfsm-like
namespace (the reference package when generating fixtures, ``torchfsm_gb300``
in the GPU tests), the same program in the oracle's vocabulary, the seeded
initial condition, dt, the step count, the integrator and the recording
interval. Sizes are small so that the FP64 oracle and the reference finish
in seconds on a CPU.
"""

from __future__ import annotations

import math
from types import SimpleNamespace

import numpy as np

from torchfsm_gb300 import initial

TWO_PI = 2.0 * math.pi


def _sin_plus_half(mesh_info, batch, channels):
    x = initial.mesh_points(mesh_info)[0]
    return (np.sin(2.0 * np.pi * x) + 0.5).reshape(1, 1, -1).repeat(batch, 0)


def _grf2(seed, n, batch=2):
    return lambda mi, b, c: initial.gaussian_random_field((n, n), b, c, initial.vorticity_spectrum, seed)


def _bl(seed, shape, kmax, rms):
    return lambda mi, b, c: initial.band_limited(shape, b, c, kmax, seed, rms)


def _grf3(seed, n):
    return lambda mi, b, c: initial.gaussian_random_field((n, n, n), b, c, initial.velocity_spectrum, seed)


def _kdv_ic(mesh_info, batch, channels):
    x = initial.mesh_points(mesh_info)[0]
    L = mesh_info[0][1] - mesh_info[0][0]
    u = 0.5 * np.cos(2 * np.pi * x / L) + 0.3 * np.sin(4 * np.pi * x / L)
    return u.reshape(1, 1, -1).repeat(batch, 0)


def _kolmogorov_source(mesh_info, batch, channels):
    # -4 cos(4 y) (forcing of the vorticity equation, sign as in field.kolm_force)
    y = initial.mesh_points(mesh_info)[1]
    f = -4.0 * np.cos(4.0 * y)
    return np.broadcast_to(f.reshape(1, 1, 1, -1), (1, 1, mesh_info[0][2], mesh_info[1][2])).copy()


CASES = {
    # The README example exactly: 1D Burgers nu = 0.01, N = 128, u0 = sin(2 pi x) + 0.5, 200 steps.
    "burgers1d_readme_n128": dict(
        mesh=[(0, 1, 128)], batch=1, channels=1, dt=0.01, step=200, record=1,
        build=lambda M: M.pde.Burgers(0.01),
        lin=[(0.01, ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_sin_plus_half,
    ),
    # 2D vorticity NS, NavierStokesVorticity(1000), on a small grid.
    "ns2d_n32": dict(
        mesh=[(0, TWO_PI, 32), (0, TWO_PI, 32)], batch=2, channels=1, dt=0.01, step=50, record=10,
        build=lambda M: M.pde.NavierStokesVorticity(1000),
        lin=[(1.0 / 1000, ("laplacian",))], nl=[(-1.0, "vorticity_convection")],
        ic=_grf2(11, 32),
    ),
    "ns2d_n64_re100": dict(
        mesh=[(0, TWO_PI, 64), (0, TWO_PI, 64)], batch=1, channels=1, dt=0.005, step=40, record=0,
        build=lambda M: M.pde.NavierStokesVorticity(100),
        lin=[(1.0 / 100, ("laplacian",))], nl=[(-1.0, "vorticity_convection")],
        ic=_grf2(12, 64),
    ),
    # 2D Burgers (two velocity channels).
    "burgers2d_n32": dict(
        mesh=[(0, TWO_PI, 32), (0, TWO_PI, 32)], batch=2, channels=2, dt=0.01, step=40, record=10,
        build=lambda M: M.pde.Burgers(0.01),
        lin=[(0.01, ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_bl(21, (32, 32), 4, 0.25),
    ),
    "burgers2d_l1_n64": dict(
        mesh=[(0, 1, 64), (0, 1, 64)], batch=1, channels=2, dt=0.001, step=30, record=0,
        build=lambda M: M.pde.Burgers(0.01),
        lin=[(0.01, ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_bl(22, (64, 64), 6, 0.5),
    ),
    # 1D Kuramoto-Sivashinsky on L = 32 pi (serving family).
    "ks1d_n128": dict(
        mesh=[(0, 32 * math.pi, 128)], batch=2, channels=1, dt=0.05, step=100, record=20,
        build=lambda M: M.pde.KuramotoSivashinsky(),
        lin=[(-1.0, ("laplacian",)), (-1.0, ("biharmonic",))], nl=[(-1.0, "convection")],
        ic=_bl(31, (128,), 8, 1.0),
    ),
    # 1D Korteweg-de Vries: odd symbol (complex E, real-part phi quirk, complex Nyquist).
    "kdv1d_n64": dict(
        mesh=[(0, 20.0, 64)], batch=1, channels=1, dt=1e-3, step=100, record=25,
        build=lambda M: M.pde.KortewegDeVries(),
        lin=[(-1.0, ("spatial_derivative", 0, 3))], nl=[(6.0, "convection")],
        ic=_kdv_ic,
    ),
    # 3D Burgers, three velocity channels.
    "burgers3d_n16": dict(
        mesh=[(0, TWO_PI, 16)] * 3, batch=1, channels=3, dt=0.01, step=10, record=0,
        build=lambda M: M.pde.Burgers(0.005),
        lin=[(0.005, ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_grf3(41, 16),
    ),
    # Linear-only program: the auto integrator is ETDRK0.
    "heat2d_etdrk0": dict(
        mesh=[(0, 1, 32), (0, 1, 32)], batch=2, channels=1, dt=0.001, step=10, record=1,
        build=lambda M: 0.05 * M.operator.Laplacian(),
        lin=[(0.05, ("laplacian",))], nl=[],
        ic=_bl(51, (32, 32), 5, 1.0),
    ),
    # Batched viscosity: a [B,1,1] tensor coefficient.
    "burgers1d_batched_nu": dict(
        mesh=[(0, 1, 64)], batch=3, channels=1, dt=0.01, step=50, record=0,
        build=lambda M: M.torch.tensor([0.01, 0.02, 0.05], dtype=M.torch.float64).reshape(3, 1, 1) * M.operator.Laplacian() - M.operator.Convection(),
        lin=[(np.array([0.01, 0.02, 0.05]).reshape(3, 1, 1), ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_bl(61, (64,), 5, 1.0),
    ),
    # High-dimensional KS: the mean removed is the mean over the whole batch.
    "ksnd2d_n32": dict(
        mesh=[(0, 10 * math.pi, 32), (0, 10 * math.pi, 32)], batch=2, channels=1, dt=0.05, step=20, record=5,
        build=lambda M: M.pde.KuramotoSivashinskyHighDim(),
        lin=[(-1.0, ("laplacian",)), (-1.0, ("biharmonic",))], nl=[(-1.0, "ks_convection")],
        ic=_bl(71, (32, 32), 4, 0.5),
    ),
    # 1D KSConvection with the mean removed over a batch of three samples.
    "ksnd1d_b3_n64": dict(
        mesh=[(0, 10 * math.pi, 64)], batch=3, channels=1, dt=0.05, step=40, record=8,
        build=lambda M: M.pde.KuramotoSivashinskyHighDim(),
        lin=[(-1.0, ("laplacian",)), (-1.0, ("biharmonic",))], nl=[(-1.0, "ks_convection")],
        ic=_bl(113, (64,), 6, 0.7),
    ),
    # Velocity-form NS with the Leray projection.
    "nsvel2d_n32": dict(
        mesh=[(0, TWO_PI, 32), (0, TWO_PI, 32)], batch=1, channels=2, dt=0.01, step=20, record=0,
        build=lambda M: M.pde.NavierStokes(100),
        lin=[(1.0 / 100, ("laplacian",))], nl=[(1.0, "ns_pressure_convection")],
        ic=_bl(81, (32, 32), 4, 0.5),
    ),
    # Vorticity NS with linear drag (unit implicit source) and an explicit Kolmogorov source.
    "ns2d_kolmogorov_n32": dict(
        mesh=[(0, TWO_PI, 32), (0, TWO_PI, 32)], batch=1, channels=1, dt=0.01, step=30, record=0,
        build=lambda M: M.pde.NavierStokesVorticity(100) + (-0.1) * M.operator.ImplicitSource() - M.operator.ExplicitSource(M.torch.tensor(4.0 * np.cos(4.0 * initial.mesh_points([(0, TWO_PI, 32), (0, TWO_PI, 32)])[1])).reshape(1, 1, 1, 32).expand(1, 1, 32, 32)),
        lin=[(1.0 / 100, ("laplacian",)), (-0.1, ("unit",))],
        nl=[(-1.0, "vorticity_convection"), (-1.0, ("source_phys", 4.0))],
        ic=_grf2(91, 32),
    ),
}

CASES.update({
    # 3D high-dimensional KS (scalar, batch-wide mean removal).
    "ksnd3d_n16": dict(
        mesh=[(0, 10 * math.pi, 16)] * 3, batch=2, channels=1, dt=0.05, step=10, record=0,
        build=lambda M: M.pde.KuramotoSivashinskyHighDim(),
        lin=[(-1.0, ("laplacian",)), (-1.0, ("biharmonic",))], nl=[(-1.0, "ks_convection")],
        ic=_bl(101, (16, 16, 16), 3, 0.5),
    ),
    # 3D velocity Navier-Stokes with the Leray projection.
    "nsvel3d_n16": dict(
        mesh=[(0, TWO_PI, 16)] * 3, batch=1, channels=3, dt=0.01, step=10, record=5,
        build=lambda M: M.pde.NavierStokes(100),
        lin=[(1.0 / 100, ("laplacian",))], nl=[(1.0, "ns_pressure_convection")],
        ic=_bl(111, (16, 16, 16), 3, 0.5),
    ),
    # 3D Burgers on 32^3, two samples.
    "burgers3d_n32": dict(
        mesh=[(0, TWO_PI, 32)] * 3, batch=2, channels=3, dt=0.005, step=8, record=0,
        build=lambda M: M.pde.Burgers(0.01),
        lin=[(0.01, ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_grf3(121, 32),
    ),
    # 2D vorticity NS on 512^2 (the largest 2D size).
    "ns2d_n512": dict(
        mesh=[(0, TWO_PI, 512), (0, TWO_PI, 512)], batch=1, channels=1, dt=1e-3, step=4, record=0,
        build=lambda M: M.pde.NavierStokesVorticity(1000),
        lin=[(1.0 / 1000, ("laplacian",))], nl=[(-1.0, "vorticity_convection")],
        ic=_grf2(131, 512),
    ),
    # 2D Burgers at the differentiable workload's size (128^2, two channels).
    "burgers2d_n128": dict(
        mesh=[(0, TWO_PI, 128), (0, TWO_PI, 128)], batch=2, channels=2, dt=0.005, step=20, record=0,
        build=lambda M: M.pde.Burgers(0.01),
        lin=[(0.01, ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_bl(141, (128, 128), 6, 1.0),
    ),
})

# Alternative integrators on the README 1D Burgers program (64 points, 50 steps).
for _name in ("setdrk1", "setdrk2", "setdrk3", "etdrk1", "etdrk2"):
    CASES[f"burgers1d_{_name}"] = dict(
        mesh=[(0, 1, 64)], batch=1, channels=1, dt=0.005, step=50, record=0,
        build=lambda M: M.pde.Burgers(0.02), integrator=_name,
        lin=[(0.02, ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_sin_plus_half,
    )

# Explicit Runge-Kutta integrators (integrator/_rk.py), fixed step: every tableau on 1D Burgers
# (32 points, so that |dt L| <= 1 stays inside every scheme's stability region), and RK on the
# other fused paths: 2D plane passes, vorticity, 3D volume passes, the linear pointwise kernel,
# and the 1D KS batch-mean fix-up.
RK_NAMES = ("Euler", "Midpoint", "Heun12", "Ralston12", "BogackiShampine23", "RK4", "RK4_38Rule", "Dorpi45",
            "Fehlberg45", "CashKarp45")
for _name in RK_NAMES:
    CASES[f"burgers1d_rk_{_name.lower()}"] = dict(
        mesh=[(0, 1, 32)], batch=2, channels=1, dt=0.005, step=50, record=10,
        build=lambda M: M.pde.Burgers(0.02), integrator=_name,
        lin=[(0.02, ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_bl(171, (32,), 4, 0.5),
    )
CASES.update({
    "burgers2d_rk4_n32": dict(
        mesh=[(0, TWO_PI, 32), (0, TWO_PI, 32)], batch=2, channels=2, dt=0.01, step=20, record=5,
        build=lambda M: M.pde.Burgers(0.01), integrator="RK4",
        lin=[(0.01, ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_bl(181, (32, 32), 4, 0.5),
    ),
    "ns2d_dorpi45_n32": dict(
        mesh=[(0, TWO_PI, 32), (0, TWO_PI, 32)], batch=2, channels=1, dt=0.01, step=20, record=0,
        build=lambda M: M.pde.NavierStokesVorticity(1000), integrator="Dorpi45",
        lin=[(1.0 / 1000, ("laplacian",))], nl=[(-1.0, "vorticity_convection")],
        ic=_grf2(191, 32),
    ),
    "burgers3d_fehlberg45_n16": dict(
        mesh=[(0, TWO_PI, 16)] * 3, batch=1, channels=3, dt=0.01, step=8, record=0,
        build=lambda M: M.pde.Burgers(0.005), integrator="Fehlberg45",
        lin=[(0.005, ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_grf3(201, 16),
    ),
    "heat2d_rk4": dict(
        mesh=[(0, 1, 32), (0, 1, 32)], batch=2, channels=1, dt=0.001, step=10, record=1,
        build=lambda M: 0.05 * M.operator.Laplacian(), integrator="RK4",
        lin=[(0.05, ("laplacian",))], nl=[],
        ic=_bl(211, (32, 32), 5, 1.0),
    ),
    "ksnd1d_b3_rk438": dict(
        mesh=[(0, 10 * math.pi, 64)], batch=3, channels=1, dt=0.001, step=40, record=8,
        build=lambda M: M.pde.KuramotoSivashinskyHighDim(), integrator="RK4_38Rule",
        lin=[(-1.0, ("laplacian",)), (-1.0, ("biharmonic",))], nl=[(-1.0, "ks_convection")],
        ic=_bl(221, (64,), 6, 0.7),
    ),
})


# Cases at the benchmarked kernel instances (the 256-point register transforms of the 2D plane
# passes and of each 3D axis, the split launch of a large 2D batch, and the 1D line kernel at the
# serving sizes). Their batches are too large to store: the fixture keeps the samples named in
# ``keep`` (final physical fields, float32) and every sample's L2 norm (float64), the GPU test
# runs the whole batch, and the oracle test integrates the ``oracle_samples`` alone (every sample
# of these programs evolves independently).
LARGE_CASES = {
    # 2D vorticity NS at the headline's grid, dt and viscosity, the first 48 of its seeded fields: a
    # batch of 48 x 256 x 129 spectral points runs split into parts on forked streams.
    "ns2d_n256_b48": dict(
        mesh=[(0, TWO_PI, 256), (0, TWO_PI, 256)], batch=48, channels=1, dt=1e-3, step=50, record=0,
        build=lambda M: M.pde.NavierStokesVorticity(1000),
        lin=[(1.0 / 1000, ("laplacian",))], nl=[(-1.0, "vorticity_convection")],
        ic=_grf2(2024, 256), keep=[0, 13, 31, 47], oracle_samples=[0],
    ),
    # 2D Burgers at the serving stream's largest grid (two velocity channels).
    "burgers2d_n256": dict(
        mesh=[(0, TWO_PI, 256), (0, TWO_PI, 256)], batch=2, channels=2, dt=0.01, step=30, record=0,
        build=lambda M: M.pde.Burgers(0.01),
        lin=[(0.01, ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_bl(251, (256, 256), 8, 0.25), keep=[1], oracle_samples=[1],
    ),
    # 3D Burgers with one axis of 256 points each: the x pass, the y passes and the z pass of the
    # 256^3 workload at their 256-point instances.
    "burgers3d_256x16x16": dict(
        mesh=[(0, TWO_PI, 256), (0, TWO_PI, 16), (0, TWO_PI, 16)], batch=1, channels=3, dt=5e-3, step=20, record=0,
        build=lambda M: M.pde.Burgers(0.005),
        lin=[(0.005, ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_bl(261, (256, 16, 16), 3, 1.0), keep=[0], oracle_samples=[0],
    ),
    "burgers3d_16x256x16": dict(
        mesh=[(0, TWO_PI, 16), (0, TWO_PI, 256), (0, TWO_PI, 16)], batch=1, channels=3, dt=5e-3, step=20, record=0,
        build=lambda M: M.pde.Burgers(0.005),
        lin=[(0.005, ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_bl(262, (16, 256, 16), 3, 1.0), keep=[0], oracle_samples=[0],
    ),
    "burgers3d_16x16x256": dict(
        mesh=[(0, TWO_PI, 16), (0, TWO_PI, 16), (0, TWO_PI, 256)], batch=1, channels=3, dt=5e-3, step=20, record=0,
        build=lambda M: M.pde.Burgers(0.005),
        lin=[(0.005, ("laplacian",))], nl=[(-1.0, "convection")],
        ic=_bl(263, (16, 16, 256), 3, 1.0), keep=[0], oracle_samples=[0],
    ),
    # 1D Kuramoto-Sivashinsky on L = 32 pi at two of the serving stream's sizes.
    "ks1d_n1024": dict(
        mesh=[(0, 32 * math.pi, 1024)], batch=3, channels=1, dt=0.05, step=200, record=0,
        build=lambda M: M.pde.KuramotoSivashinsky(),
        lin=[(-1.0, ("laplacian",)), (-1.0, ("biharmonic",))], nl=[(-1.0, "convection")],
        ic=_bl(271, (1024,), 8, 1.0), keep=[0, 1, 2], oracle_samples=[0, 1, 2],
    ),
    "ks1d_n4096": dict(
        mesh=[(0, 32 * math.pi, 4096)], batch=3, channels=1, dt=0.02, step=200, record=0,
        build=lambda M: M.pde.KuramotoSivashinsky(),
        lin=[(-1.0, ("laplacian",)), (-1.0, ("biharmonic",))], nl=[(-1.0, "convection")],
        ic=_bl(272, (4096,), 8, 1.0), keep=[0, 1, 2], oracle_samples=[0, 1, 2],
    ),
}


def _allen_cahn_source(u):
    return u - u ** 3


def _damping_source(u):
    return -0.5 * u * u.abs()


def _burgers_with_sources(M):
    x = M.torch.arange(64, dtype=M.torch.float64) / 64
    forcing = (0.1 * M.torch.sin(2 * math.pi * x)).reshape(1, 1, 64)
    return M.pde.Burgers(0.02) + M.operator.ImplicitSource(_damping_source) + forcing


# Programs without a fused kernel (Python-callable sources, the conservative convection form, two
# kinds of nonlinear term with an explicit source): integrate steps them through the cores'
# Python callables with the library's coefficient tables and transforms.
CALLBACK_CASES = {
    "allencahn1d_n64": dict(
        mesh=[(0, TWO_PI, 64)], batch=2, channels=1, dt=0.01, step=100, record=20,
        build=lambda M: 0.05 * M.operator.Laplacian() + M.operator.ImplicitSource(_allen_cahn_source),
        ic=_bl(231, (64,), 4, 0.5),
    ),
    "allencahn1d_setdrk2": dict(
        mesh=[(0, TWO_PI, 64)], batch=2, channels=1, dt=0.01, step=50, record=0, integrator="setdrk2",
        build=lambda M: 0.05 * M.operator.Laplacian() + M.operator.ImplicitSource(_allen_cahn_source),
        ic=_bl(232, (64,), 4, 0.5),
    ),
    "allencahn1d_setdrk3_raw": dict(
        mesh=[(0, TWO_PI, 64)], batch=1, channels=1, dt=0.01, step=50, record=0, integrator="setdrk3",
        build=lambda M: 0.05 * M.operator.Laplacian()
        + M.operator.ImplicitSource(_allen_cahn_source, non_linear=False),
        ic=_bl(233, (64,), 4, 0.5),
    ),
    "allencahn1d_etdrk2": dict(
        mesh=[(0, TWO_PI, 64)], batch=2, channels=1, dt=0.01, step=50, record=10, integrator="etdrk2",
        build=lambda M: 0.05 * M.operator.Laplacian() + M.operator.ImplicitSource(_allen_cahn_source),
        ic=_bl(234, (64,), 4, 0.5),
    ),
    "conservative_burgers2d_n32": dict(
        mesh=[(0, TWO_PI, 32), (0, TWO_PI, 32)], batch=2, channels=2, dt=0.01, step=30, record=10,
        build=lambda M: 0.01 * M.operator.Laplacian() - M.operator.ConservativeConvection(),
        ic=_bl(235, (32, 32), 4, 0.25),
    ),
    "burgers1d_sources_n64": dict(
        mesh=[(0, 1, 64)], batch=2, channels=1, dt=0.005, step=60, record=15,
        build=_burgers_with_sources,
        ic=_bl(236, (64,), 4, 0.5),
    ),
}


def _case(name: str) -> dict:
    for table in (CASES, LARGE_CASES, CALLBACK_CASES):
        if name in table:
            return table[name]
    raise KeyError(name)


def set_case_integrator(op, M, kind):
    """Select a case's integrator by name on a torchfsm-like namespace."""
    if kind in RK_NAMES:
        op.set_integrator(M.integrator.RKIntegrator[kind])
    elif kind.startswith("setdrk"):
        op.set_integrator(M.integrator.SETDRKIntegrator[kind.upper()])
    else:
        op.set_integrator(M.integrator.ETDRKIntegrator[kind.upper()])


def initial_condition(name: str) -> np.ndarray:
    c = _case(name)
    return np.ascontiguousarray(c["ic"](c["mesh"], c["batch"], c["channels"]), dtype=np.float64)


def record_fn(name: str):
    every = _case(name)["record"]
    if not every:
        return None
    return lambda step: step % every == 0


def oracle_terms(name: str):
    """Linear and nonlinear term lists in the oracle's vocabulary (sources resolved to spectra)."""
    c = _case(name)
    nl = []
    for coef, spec in c["nl"]:
        if isinstance(spec, tuple) and spec[0] == "source_phys":
            y = initial.mesh_points(c["mesh"])[1]
            f = spec[1] * np.cos(spec[1] * y)
            f = np.broadcast_to(f.reshape(1, 1, 1, -1), (1, 1, c["mesh"][0][2], c["mesh"][1][2]))
            nl.append((coef, ("source", np.fft.fftn(f, axes=(-2, -1)))))
        else:
            nl.append((coef, spec))
    return c["lin"], nl


def namespace(module_root):
    """torchfsm-like namespace (``pde``, ``operator``, ``torch``) from a package root module."""
    import importlib
    import torch

    return SimpleNamespace(
        pde=importlib.import_module(module_root + ".pde"),
        operator=importlib.import_module(module_root + ".operator"),
        integrator=importlib.import_module(module_root + ".integrator"),
        functional=importlib.import_module(module_root + ".functional"),
        traj_recorder=importlib.import_module(module_root + ".traj_recorder"),
        torch=torch,
    )


# Differentiable workloads: loss = MSE(u_T(u0, nu), target), target from the same u0 with nu_target.
GRAD_CASES = {
    "grad_burgers2d_n32": dict(
        mesh=[(0, TWO_PI, 32), (0, TWO_PI, 32)], batch=2, channels=2, dt=0.005, step=20,
        nu=0.01, nu_target=0.02, ic=_bl(151, (32, 32), 4, 1.0),
    ),
    "grad_burgers1d_n64": dict(
        mesh=[(0, TWO_PI, 64)], batch=3, channels=1, dt=0.01, step=30,
        nu=0.05, nu_target=0.1, ic=_bl(161, (64,), 5, 1.0),
    ),
}


# Differentiable programs the hand-written Convection adjoint does not cover (their gradients come
# from segments recomputed in torch arithmetic and differentiated by autograd): vorticity NS, the
# high-dimensional KS (batch-wide mean), KdV (complex symbol). build(M, coef) makes the operator with
# the tensor coefficient ``coef`` on its first linear term; the target is the run with coef_target.
GENERIC_GRAD_CASES = {
    "grad_ns2d_n32": dict(
        mesh=[(0, TWO_PI, 32), (0, TWO_PI, 32)], batch=2, channels=1, dt=0.01, step=20, coef=0.01,
        coef_target=0.02, ic=_grf2(301, 32),
        build=lambda M, c: c * M.operator.Laplacian() - M.operator.VorticityConvection(),
    ),
    "grad_ksnd2d_n32": dict(
        mesh=[(0, 10 * math.pi, 32), (0, 10 * math.pi, 32)], batch=2, channels=1, dt=0.02, step=15, coef=-1.0,
        coef_target=-1.2, ic=_bl(302, (32, 32), 4, 0.5),
        build=lambda M, c: c * M.operator.Laplacian() - M.operator.Biharmonic() - M.operator.KSConvection(),
    ),
    "grad_kdv1d_n64": dict(
        mesh=[(0, 20.0, 64)], batch=2, channels=1, dt=1e-3, step=30, coef=-1.0, coef_target=-1.1,
        ic=_bl(303, (64,), 4, 0.5),
        build=lambda M, c: c * M.operator.SpatialDerivative(0, 3) + 6.0 * M.operator.Convection(),
    ),
    # other integrators: the recomputed segments step with the scheme's own recurrence and tables
    "grad_burgers1d_etdrk2_n64": dict(
        mesh=[(0, TWO_PI, 64)], batch=2, channels=1, dt=0.01, step=30, coef=0.05, coef_target=0.08,
        ic=_bl(304, (64,), 4, 0.5), integrator="etdrk2",
        build=lambda M, c: c * M.operator.Laplacian() - M.operator.Convection(),
    ),
    "grad_burgers2d_setdrk3_n32": dict(
        mesh=[(0, TWO_PI, 32), (0, TWO_PI, 32)], batch=2, channels=2, dt=0.01, step=20, coef=0.05,
        coef_target=0.08, ic=_bl(305, (32, 32), 4, 0.5), integrator="setdrk3",
        build=lambda M, c: c * M.operator.Laplacian() - M.operator.Convection(),
    ),
    "grad_burgers1d_rk4_n64": dict(
        mesh=[(0, TWO_PI, 64)], batch=2, channels=1, dt=0.005, step=30, coef=0.05, coef_target=0.08,
        ic=_bl(306, (64,), 4, 0.5), integrator="RK4",
        build=lambda M, c: c * M.operator.Laplacian() - M.operator.Convection(),
    ),
    "grad_heat2d_etdrk0_n16": dict(
        mesh=[(0, TWO_PI, 16), (0, TWO_PI, 16)], batch=2, channels=1, dt=0.05, step=10, coef=0.1,
        coef_target=0.15, ic=_bl(307, (16, 16), 4, 1.0),
        build=lambda M, c: c * M.operator.Laplacian(),
    ),
}


def build_generic_grad_op(name: str, M, coef):
    """The operator of a generic gradient case with its coefficient and integrator."""
    case = GENERIC_GRAD_CASES[name]
    op = case["build"](M, coef)
    if case.get("integrator"):
        set_case_integrator(op, M, case["integrator"])
    return op


def generic_grad_initial_condition(name: str) -> np.ndarray:
    c = GENERIC_GRAD_CASES[name]
    return np.ascontiguousarray(c["ic"](c["mesh"], c["batch"], c["channels"]), dtype=np.float64)


def grad_initial_condition(name: str) -> np.ndarray:
    c = GRAD_CASES[name]
    return np.ascontiguousarray(c["ic"](c["mesh"], c["batch"], c["channels"]), dtype=np.float64)


# One-shot evaluation (Operator.__call__, LinearOperator.solve, functional.*): fn(M, u, mesh) on a
# float64 field; programs the library lowers run fused (the FSM_APPLY scheme), the
# channel-changing post-processing cores through torch spectral multiplies.
APPLY_CASES = {
    "apply_burgers2d_n32": dict(mesh=[(0, TWO_PI, 32)] * 2, ic=_bl(231, (32, 32), 6, 1.0), batch=2, channels=2,
                                fn=lambda M, u, m: M.pde.Burgers(0.01)(u=u, mesh=m), fused=True,
        lin=[(0.01, ("laplacian",))], nl=[(-1.0, "convection")]),
    "apply_ns2d_n32": dict(mesh=[(0, TWO_PI, 32)] * 2, ic=_bl(232, (32, 32), 6, 1.0), batch=2, channels=1,
                           fn=lambda M, u, m: M.pde.NavierStokesVorticity(100)(u=u, mesh=m), fused=True,
        lin=[(1.0 / 100, ("laplacian",))], nl=[(-1.0, "vorticity_convection")]),
    "apply_ksnd2d_n32": dict(mesh=[(0, 10 * math.pi, 32)] * 2, ic=_bl(233, (32, 32), 4, 0.5), batch=2, channels=1,
                             fn=lambda M, u, m: M.pde.KuramotoSivashinskyHighDim()(u=u, mesh=m), fused=True,
        lin=[(-1.0, ("laplacian",)), (-1.0, ("biharmonic",))], nl=[(-1.0, "ks_convection")]),
    "apply_nsvel2d_n32": dict(mesh=[(0, TWO_PI, 32)] * 2, ic=_bl(234, (32, 32), 6, 1.0), batch=1, channels=2,
                              fn=lambda M, u, m: M.pde.NavierStokes(100)(u=u, mesh=m), fused=True,
        lin=[(1.0 / 100, ("laplacian",))], nl=[(1.0, "ns_pressure_convection")]),
    "apply_kdv1d_n64": dict(mesh=[(0, 20.0, 64)], ic=_bl(235, (64,), 5, 1.0), batch=2, channels=1,
                            fn=lambda M, u, m: M.pde.KortewegDeVries()(u=u, mesh=m), fused=True,
        lin=[(-1.0, ("spatial_derivative", 0, 3))], nl=[(6.0, "convection")]),
    "apply_burgers3d_n16": dict(mesh=[(0, TWO_PI, 16)] * 3, ic=_bl(236, (16, 16, 16), 3, 1.0), batch=1, channels=3,
                                fn=lambda M, u, m: M.pde.Burgers(0.005)(u=u, mesh=m), fused=True,
        lin=[(0.005, ("laplacian",))], nl=[(-1.0, "convection")]),
    "apply_heat2d_n32": dict(mesh=[(0, 1, 32)] * 2, ic=_bl(237, (32, 32), 5, 1.0), batch=2, channels=1,
                             fn=lambda M, u, m: (0.05 * M.operator.Laplacian())(u=u, mesh=m), fused=True,
        lin=[(0.05, ("laplacian",))], nl=[]),
    "apply_grad_n32": dict(mesh=[(0, TWO_PI, 32)] * 2, ic=_bl(238, (32, 32), 6, 1.0), batch=2, channels=1,
                           fn=lambda M, u, m: M.functional.grad(u, mesh=m)),
    "apply_div_n32": dict(mesh=[(0, TWO_PI, 32)] * 2, ic=_bl(239, (32, 32), 6, 1.0), batch=2, channels=2,
                          fn=lambda M, u, m: M.functional.div(u, mesh=m)),
    "apply_curl2d_n32": dict(mesh=[(0, TWO_PI, 32)] * 2, ic=_bl(240, (32, 32), 6, 1.0), batch=2, channels=2,
                             fn=lambda M, u, m: M.functional.curl(u, mesh=m)),
    "apply_curl3d_n16": dict(mesh=[(0, TWO_PI, 16)] * 3, ic=_bl(241, (16, 16, 16), 3, 1.0), batch=1, channels=3,
                             fn=lambda M, u, m: M.functional.curl(u, mesh=m)),
    "apply_vort2vel_n32": dict(mesh=[(0, TWO_PI, 32)] * 2, ic=_bl(242, (32, 32), 6, 1.0), batch=2, channels=1,
                               fn=lambda M, u, m: M.functional.vorticity2velocity(u, mesh=m)),
    "apply_vort2press_n32": dict(mesh=[(0, TWO_PI, 32)] * 2, ic=_bl(243, (32, 32), 6, 1.0), batch=2, channels=1,
                                 fn=lambda M, u, m: M.functional.vorticity2pressure(u, mesh=m)),
    "apply_vel2press_n32": dict(mesh=[(0, TWO_PI, 32)] * 2, ic=_bl(244, (32, 32), 6, 1.0), batch=2, channels=2,
                                fn=lambda M, u, m: M.functional.velocity2pressure(u, mesh=m)),
    "apply_vort2press_op_n32": dict(mesh=[(0, TWO_PI, 32)] * 2, ic=_bl(245, (32, 32), 6, 1.0), batch=2, channels=1,
                                    fn=lambda M, u, m: M.operator.Vorticity2Pressure()(u=u, mesh=m)),
    "apply_vel2press_op_n32": dict(mesh=[(0, TWO_PI, 32)] * 2, ic=_bl(246, (32, 32), 6, 1.0), batch=2, channels=2,
                                   fn=lambda M, u, m: M.operator.Velocity2Pressure()(u=u, mesh=m)),
    "apply_laplacian_fn_n32": dict(mesh=[(0, TWO_PI, 32)] * 2, ic=_bl(247, (32, 32), 6, 1.0), batch=2, channels=1,
                                   fn=lambda M, u, m: M.functional.laplacian(u, mesh=m), fused=True,
        lin=[(1.0, ("laplacian",))], nl=[]),
    "apply_convection_fn_n32": dict(mesh=[(0, TWO_PI, 32)] * 2, ic=_bl(248, (32, 32), 6, 1.0), batch=2, channels=2,
                                    fn=lambda M, u, m: M.functional.convection(u, mesh=m), fused=True,
        lin=[], nl=[(1.0, "convection")]),
    "apply_solve_biharmonic_n32": dict(mesh=[(0, TWO_PI, 32)] * 2, ic=_bl(249, (32, 32), 6, 1.0), batch=2, channels=1,
                                       fn=lambda M, u, m: M.operator.Biharmonic().solve(u, mesh=m, n_channel=1)),
}


def apply_input(name: str) -> np.ndarray:
    c = APPLY_CASES[name]
    return np.ascontiguousarray(c["ic"](c["mesh"], c["batch"], c["channels"]), dtype=np.float64)
