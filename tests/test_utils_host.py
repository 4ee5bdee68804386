"""Trajectory helpers and API names with the reference's behaviour (no GPU): outputs pinned to
the reference's own outputs (tests/golden/make_utils_golden.py), numpy inputs, type aliases,
package-root re-exports."""

import os
from typing import Annotated, List, Union

import numpy as np
import pytest
import torch

import torchfsm_gb300 as fsm
from torchfsm_gb300 import utils as U
from torchfsm_gb300._type import FourierArray, FourierTensor, SpatialArray, SpatialTensor, ValueList

GOLDEN = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "utils_helpers.npz"))
CALLS = [("random_clip_traj", 5), ("random_select_frames", 7), ("uniformly_select_frames", 6)]


@pytest.mark.parametrize("name,arg", CALLS)
@pytest.mark.parametrize("seed", [3, 11])
def test_frame_helpers_match_reference(name, arg, seed):
    x = GOLDEN["traj"]
    torch.manual_seed(seed)
    got = getattr(U, name)(torch.from_numpy(x), arg)
    assert np.array_equal(got.numpy(), GOLDEN[f"{name}_{seed}"])
    # numpy input: same frames, returned as a tensor (as the reference does)
    torch.manual_seed(seed)
    got_np = getattr(U, name)(x, arg)
    assert isinstance(got_np, torch.Tensor) and np.array_equal(got_np.numpy(), GOLDEN[f"{name}_{seed}"])


def test_statistics_match_reference():
    x = GOLDEN["traj"]
    means, stds, mins, maxs = U.statistics_traj([torch.from_numpy(x), x[:2, 5:]])
    for got, key in [(means, "mean"), (stds, "std"), (mins, "min"), (maxs, "max")]:
        assert np.allclose(got, GOLDEN[f"stats_{key}"], rtol=1e-6, atol=1e-7)


def test_type_aliases():
    assert SpatialTensor["B C H"] == Annotated[torch.Tensor, "B C H"]
    assert FourierTensor["B C H"] == Annotated[torch.Tensor, "B C H"]
    assert SpatialArray["B"] == Annotated[np.ndarray, "B"] and FourierArray["B"] == Annotated[np.ndarray, "B"]
    assert ValueList[int] == Union[int, List[int]]
    with pytest.raises(TypeError):
        SpatialTensor()


def test_package_root_reexports_the_operator_algebra():
    for name in ("Laplacian", "Biharmonic", "Convection", "VorticityConvection", "KSConvection",
                 "NSPressureConvection", "SpatialDerivative", "ImplicitSource", "ExplicitSource", "Grad", "Div",
                 "Curl", "LinearOperator", "NonlinearOperator", "run_operators", "MeshGrid", "FourierMesh"):
        assert hasattr(fsm, name), name
    op = fsm.Laplacian() * 0.1 - fsm.Convection()
    assert isinstance(op, fsm.Operator)


def test_fused_programs_need_cuda_inputs():
    """Programs the library covers never evaluate on the CPU; channel-changing post-processing
    cores (not lowered) evaluate with torch on the input's device."""
    import math

    from torchfsm_gb300 import pde

    mesh = [(0, 2 * math.pi, 16)] * 2
    with pytest.raises(RuntimeError, match="CUDA"):
        pde.NavierStokesVorticity(100)(u=torch.randn(1, 1, 16, 16), mesh=mesh)
    with pytest.raises(RuntimeError, match="CUDA"):
        pde.Burgers(0.01).integrate(u_0=torch.randn(1, 2, 16, 16), mesh=mesh, dt=0.01, step=2)
    assert fsm.Div()(u=torch.randn(1, 2, 16, 16), mesh=mesh).shape == (1, 1, 16, 16)


def test_format_device_dtype():
    import torch

    # the reference's rules: no device -> CPU, "cuda" -> cuda:0, no dtype -> float32
    assert U.format_device_dtype() == (torch.device("cpu"), torch.float32)
    assert U.format_device_dtype("cuda") == (torch.device("cuda", 0), torch.float32)
    assert U.format_device_dtype("cuda:1", torch.float64) == (torch.device("cuda", 1), torch.float64)
    assert U.format_device_dtype("cpu")[0] == torch.device("cpu")
    # a device object without an index is given index 0 as well, so that a mesh's device compares
    # equal to its tensors' (the reference leaves such objects unchanged)
    assert U.format_device_dtype(torch.device("cuda"))[0] == torch.device("cuda", 0)
    assert U.default(None, 3) == 3 and U.default(0, 3) == 0
