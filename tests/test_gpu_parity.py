"""GPU parity: the fused CUDA path against the reference's FP64 runs (golden vectors).

Every case is driven through the public API (``Operator.integrate`` with the
reference's arguments), which calls the C ABI. Tolerance: relative L2 error
<= 1e-5 against the reference's float64 result, over the whole recorded
trajectory where one is recorded.
"""

import os

import numpy as np
import pytest
import torch

import cases as C
from oracle import spectral as S
from torchfsm_gb300 import _lib

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-5
pytestmark = pytest.mark.gpu

SUPPORTED = sorted(C.CASES)


def _run(name, device="cuda", dtype=torch.float32):
    case = C._case(name)
    M = C.namespace("torchfsm_gb300")
    op = case["build"](M)
    if case.get("integrator"):
        C.set_case_integrator(op, M, case["integrator"])
    u0 = torch.tensor(C.initial_condition(name), dtype=dtype, device=device)
    rec_fn = C.record_fn(name)
    rec = M.traj_recorder.AutoRecorder(control_func=rec_fn) if rec_fn is not None else None
    out = op.integrate(u_0=u0, mesh=case["mesh"], dt=case["dt"], step=case["step"], trajectory_recorder=rec)
    return out


@pytest.mark.parametrize("name", SUPPORTED)
def test_matches_reference_fp64(name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    out = _run(name).cpu().numpy()
    ref = g["traj"] if "traj" in g else g["final"]
    assert out.shape == ref.shape
    err = S.rel_l2(out, ref)
    print(f"{name}: rel-L2 {err:.3e}")
    assert err <= TOL, f"{name}: rel-L2 {err:.3e} > {TOL}"


@pytest.mark.parametrize("name", sorted(C.LARGE_CASES))
def test_benchmarked_instances_match_reference_fp64(name):
    """The whole batch through the public API; the fixture's kept samples against the reference's
    FP64 fields and every sample's L2 norm against the reference's (the whole batch at once: a
    wrongly handled part of a split launch shows in its samples' norms)."""
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    out = _run(name).cpu().numpy().astype(np.float64)
    keep = g["keep"]
    ref = g["final_kept"].astype(np.float64)
    assert out.shape[0] == g["norms"].shape[0] and out[keep].shape == ref.shape
    err = max(S.rel_l2(out[k], ref[i]) for i, k in enumerate(keep))
    norms = np.sqrt((out.reshape(out.shape[0], -1) ** 2).sum(axis=1))
    norm_err = float(np.max(np.abs(norms - g["norms"]) / g["norms"]))
    print(f"{name}: rel-L2 {err:.3e} (kept samples), worst relative norm error {norm_err:.3e}")
    assert err <= TOL, f"{name}: rel-L2 {err:.3e} > {TOL}"
    assert norm_err <= TOL, f"{name}: norm error {norm_err:.3e} > {TOL}"


def test_deterministic():
    a = _run("ns2d_n32")
    b = _run("ns2d_n32")
    assert torch.equal(a, b)


def test_python_callable_source_with_runge_kutta_is_reported_unsupported():
    M = C.namespace("torchfsm_gb300")
    op = M.operator.Laplacian() + M.operator.ImplicitSource(lambda u: u ** 2)
    op.set_integrator(M.integrator.RKIntegrator.RK4)
    u0 = torch.rand(1, 1, 64, device="cuda")
    with pytest.raises(_lib.UnsupportedProgram):
        op.integrate(u_0=u0, mesh=[(0, 1, 64)], dt=0.01, step=2)


def test_3d_axis_above_256_is_reported_unsupported():
    M = C.namespace("torchfsm_gb300")
    u0 = torch.rand(1, 3, 16, 16, 512, device="cuda")
    with pytest.raises(_lib.UnsupportedProgram):
        M.pde.Burgers(0.01).integrate(u_0=u0, mesh=[(0, 1, 16), (0, 1, 16), (0, 1, 512)], dt=0.01, step=1)
