"""``Operator.integrate``'s arguments and state handling, on the CPU.

Mesh given as a list, a MeshGrid or a FourierMesh; a registered mesh reused by later calls; a
new dt rebuilding the integrator; ``set_de_aliasing_rate``; ``set_integrator`` with the contour
options (M, r). The programs run through the callback path on the CPU stand-ins of
``tests/cpu_library.py`` (the integrate driver, the callback plan and the conversions are the
product's own code) and are compared with each other or with the FP64 oracle at the parity bar.
"""

import math

import numpy as np
import pytest
import torch

import cpu_library as CL
from oracle import spectral as S
from torchfsm_gb300 import initial, pde
from torchfsm_gb300.integrator import SETDRKIntegrator
from torchfsm_gb300.mesh import FourierMesh, MeshGrid

TOL = 1e-5
MESH = [(0.0, 2 * math.pi, 64)]


@pytest.fixture(autouse=True)
def callback_everywhere(monkeypatch):
    CL.force_callback(monkeypatch)


def _u0(batch=2, seed=5):
    return initial.band_limited((64,), batch, 1, 4, seed, 0.5)


def _run(op, u0, **kw):
    return op.integrate(u_0=torch.tensor(u0, dtype=torch.float32), **kw).numpy()


def test_mesh_as_list_meshgrid_or_fouriermesh():
    u0 = _u0()
    a = _run(pde.Burgers(0.02), u0, mesh=MESH, dt=0.01, step=30)
    b = _run(pde.Burgers(0.02), u0, mesh=MeshGrid(MESH), dt=0.01, step=30)
    c = _run(pde.Burgers(0.02), u0, mesh=FourierMesh(MESH), dt=0.01, step=30)
    assert np.array_equal(a, b) and np.array_equal(a, c)


def test_registered_mesh_is_reused_and_a_new_dt_rebuilds():
    u0 = _u0()
    op = pde.Burgers(0.02)
    first = _run(op, u0, mesh=MESH, dt=0.01, step=30)
    again = _run(op, u0, dt=0.01, step=30)  # no mesh: the registered one
    assert np.array_equal(first, again)
    other_dt = _run(op, u0, dt=0.005, step=60)
    fresh = _run(pde.Burgers(0.02), u0, mesh=MESH, dt=0.005, step=60)
    assert op._state_dict["integrator"].dt == 0.005
    assert np.array_equal(other_dt, fresh)


@pytest.mark.parametrize("rate", [0.5, 1.0])
def test_de_aliasing_rate(rate):
    u0 = _u0()
    op = pde.Burgers(0.02)
    op.set_de_aliasing_rate(rate)
    got = _run(op, u0, mesh=MESH, dt=0.01, step=30)
    ref, _ = S.integrate(u0, MESH, [(0.02, ("laplacian",))], [(-1.0, "convection")], 0.01, 30,
                         de_aliasing_rate=rate)
    assert S.rel_l2(got, ref) <= TOL
    default, _ = S.integrate(u0, MESH, [(0.02, ("laplacian",))], [(-1.0, "convection")], 0.01, 30)
    assert S.rel_l2(ref, default) > 1e-4  # the rate matters for this field


def test_contour_options_of_set_integrator():
    u0 = _u0()
    op = pde.KuramotoSivashinsky()
    op.set_integrator(SETDRKIntegrator.SETDRK4, n_integration_points=32, integration_radius=2.0)
    mesh = [(0.0, 32 * math.pi, 64)]
    got = _run(op, u0, mesh=mesh, dt=0.05, step=40)
    ref, _ = S.integrate(u0, mesh, [(-1.0, ("laplacian",)), (-1.0, ("biharmonic",))], [(-1.0, "convection")], 0.05,
                         40, n_integration_points=32, integration_radius=2.0)
    assert S.rel_l2(got, ref) <= TOL


@pytest.mark.parametrize("fourier", [False, True])
def test_empty_batch_returns_empty_results(fourier):
    from torchfsm_gb300 import traj_recorder as TR

    u0 = torch.zeros(0, 1, 64)
    out = pde.Burgers(0.02).integrate(u_0=u0, mesh=MESH, dt=0.01, step=10, return_in_fourier=fourier)
    assert out.shape == (0, 1, 64) and out.dtype == (torch.complex64 if fourier else torch.float32)
    traj = pde.Burgers(0.02).integrate(u_0=u0.double(), mesh=MESH, dt=0.01, step=10,
                                       trajectory_recorder=TR.AutoRecorder(TR.IntervalController(5)),
                                       return_in_fourier=fourier)
    assert traj.shape == (0, 3, 1, 64) and traj.dtype == (torch.complex128 if fourier else torch.float64)
    u2 = torch.zeros(0, 2, 16, 16)
    out2 = pde.Burgers(0.02).integrate(u_0=u2, mesh=[(0, 1, 16)] * 2, dt=0.01, step=3)
    assert out2.shape == (0, 2, 16, 16)


def test_user_cores_through_the_plugin_points():
    """A user LinearCoef (here nu * Laplacian written by hand) and a user NonlinearFunc (the
    convection term written by hand) integrate like the built-in Burgers operator."""
    from torchfsm_gb300.operator import LinearCoef, NonlinearFunc, Operator

    class Diffusion(LinearCoef):
        def __call__(self, f_mesh, n_channel):
            return 0.02 * f_mesh.laplacian()

    class Advection(NonlinearFunc):
        def __call__(self, u_fft, f_mesh, u=None):
            u = f_mesh.ifft(u_fft).real if u is None else u
            return -f_mesh.fft(u * f_mesh.ifft(f_mesh.grad(0, 1) * u_fft).real)

    u0 = _u0()
    custom = Operator([lambda f_mesh, n: Diffusion(), lambda f_mesh, n: Advection()])
    got = _run(custom, u0, mesh=MESH, dt=0.01, step=30)
    ref, _ = S.integrate(u0, MESH, [(0.02, ("laplacian",))], [(-1.0, "convection")], 0.01, 30)
    assert S.rel_l2(got, ref) <= TOL
