"""Operator algebra -> spectral program lowering (CPU only)."""

import math

import numpy as np
import pytest
import torch

import cases as C
from oracle import spectral as S
from torchfsm_gb300 import _lib, _native, pde
from torchfsm_gb300.mesh import FourierMesh
from torchfsm_gb300.operator import Convection, ExplicitSource, ImplicitSource, KSConvection, Laplacian


def _register(op, mesh_info, channels, dtype=torch.float32):
    op.register_mesh(FourierMesh(mesh_info, dtype=dtype), channels)
    return op


def test_burgers_lowers_to_convection():
    op = _register(pde.Burgers(0.01), [(0, 1, 64)], 1)
    prog = _native.lower(op._linear_terms, op._nonlinear_funcs, op._state_dict["f_mesh"], 1, 2 / 3)
    assert prog.nonlinear == _lib.FSM_NL_CONVECTION and prog.nonlinear_coef == -1.0
    assert not op.is_linear


def test_ns_vorticity_lowers_to_vorticity():
    op = _register(pde.NavierStokesVorticity(1000), [(0, 2 * math.pi, 32)] * 2, 1)
    prog = _native.lower(op._linear_terms, op._nonlinear_funcs, op._state_dict["f_mesh"], 1, 2 / 3)
    assert prog.nonlinear == _lib.FSM_NL_VORTICITY and prog.nonlinear_coef == -1.0


def test_same_kind_terms_merge_and_mixed_kinds_are_rejected():
    op = _register(Laplacian() - Convection() - 0.5 * Convection(), [(0, 1, 64)], 1)
    prog = _native.lower(op._linear_terms, op._nonlinear_funcs, op._state_dict["f_mesh"], 1, 2 / 3)
    assert prog.nonlinear_coef == -1.5
    op2 = _register(Laplacian() - Convection() - KSConvection(), [(0, 1, 64)], 1)
    with pytest.raises(_lib.UnsupportedProgram):
        _native.lower(op2._linear_terms, op2._nonlinear_funcs, op2._state_dict["f_mesh"], 1, 2 / 3)


def test_python_callable_source_is_unsupported():
    op = _register(Laplacian() + ImplicitSource(lambda u: u ** 2), [(0, 1, 64)], 1)
    with pytest.raises(_lib.UnsupportedProgram):
        _native.lower(op._linear_terms, op._nonlinear_funcs, op._state_dict["f_mesh"], 1, 2 / 3)


def test_explicit_source_and_ks_flags():
    src = torch.ones(1, 1, 64)
    op = _register(Laplacian() + ExplicitSource(src), [(0, 1, 64)], 1)
    prog = _native.lower(op._linear_terms, op._nonlinear_funcs, op._state_dict["f_mesh"], 1, 2 / 3)
    assert prog.nonlinear == _lib.FSM_NL_NONE and len(prog.sources) == 1 and prog.has_nonlinear
    op2 = _register(pde.KuramotoSivashinskyHighDim(), [(0, 10.0, 32)] * 2, 1)
    prog2 = _native.lower(op2._linear_terms, op2._nonlinear_funcs, op2._state_dict["f_mesh"], 1, 2 / 3)
    assert prog2.nonlinear == _lib.FSM_NL_KS and prog2.flags & _lib.FSM_FLAG_REMOVE_MEAN


@pytest.mark.parametrize("n", [16, 48, 64, 96, 128, 256])
def test_axis_keep_matches_oracle_mask(n):
    fm = FourierMesh([(0, 2 * math.pi, n)], dtype=torch.float32)
    keep = fm.axis_keep(2 / 3)[0].numpy().astype(np.float32)
    ref = S.OMesh([(0, 2 * math.pi, n)], np.float32).low_pass_filter(2 / 3).reshape(-1)
    np.testing.assert_array_equal(keep, ref)


@pytest.mark.parametrize("name", ["ks1d_n128", "ns2d_kolmogorov_n32", "burgers1d_batched_nu", "kdv1d_n64"])
def test_linear_symbol_fp64_matches_oracle(name):
    case = C.CASES[name]
    M = C.namespace("torchfsm_gb300")
    op = case["build"](M)
    _register(op, case["mesh"], case["channels"])
    L = op._linear_coef64("cpu").numpy()
    ref = S.linear_symbol(S.OMesh(case["mesh"]), case["lin"], case["channels"])
    L = np.broadcast_to(L, np.broadcast_shapes(L.shape, ref.shape))
    np.testing.assert_allclose(L, np.broadcast_to(ref, L.shape), rtol=1e-12, atol=1e-9)


def test_rk_integrators_select_fixed_step_schemes_and_refuse_adaptive():
    from torchfsm_gb300 import pde
    from torchfsm_gb300.integrator import RKIntegrator

    op = pde.Burgers(0.01)
    for member in RKIntegrator:
        op.set_integrator(member)
        assert op._integrator_id() == member.value
        assert _lib.FSM_RK_EULER <= member.value <= _lib.FSM_RK_CASHKARP45
    op.set_integrator(RKIntegrator.Dorpi45, adaptive=True, atol=1e-6, rtol=1e-5)
    with pytest.raises(NotImplementedError):
        op._integrator_id()
