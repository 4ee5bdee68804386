"""Generate tests/golden/algebra_reference.npz: operator expressions built with the reference's
algebra (torchfsm/operator/_base.py:170-206, 826-1028) and evaluated once, in float64 on the CPU.

    python tests/golden/make_algebra_golden.py <reference source tree>

``EXPRESSIONS`` lists each expression as a name, a mesh, the input field's channels and a function
of a torchfsm-like namespace returning the operator; the file holds the reference's result of
``op(u=u, mesh=mesh)``, or the name of the exception the expression raised (building or applying
it). ``tests/test_algebra_host.py`` builds the same expressions with torchfsm_gb300.
"""

from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

M1 = [(0.0, 2 * math.pi, 32)]
M2 = [(0.0, 2 * math.pi, 16), (0.0, 2 * math.pi, 16)]


def _src(M, shape):
    x = M.torch.arange(shape[-1], dtype=M.torch.float64) / shape[-1] * 2 * math.pi
    return (M.torch.cos(x) * 0.3).reshape((1, 1) + (1,) * (len(shape) - 1) + (shape[-1],))


EXPRESSIONS = [
    ("scaled_difference", M1, 1, lambda M: (M.operator.Laplacian() - 2 * M.operator.Convection()) / 4),
    ("plus_tensor", M1, 1, lambda M: -M.operator.Laplacian() + _src(M, (32,))),
    ("tensor_plus", M1, 1, lambda M: _src(M, (32,)) + M.operator.Laplacian()),
    ("mixed_scalars", M1, 1, lambda M: 0.5 * M.operator.Laplacian() - M.operator.Biharmonic() * 0.1),
    ("negated_sum", M1, 1, lambda M: -(M.operator.Laplacian() + M.operator.Convection())),
    ("tensor_scalar_coef", M1, 1, lambda M: M.operator.Convection() * M.torch.tensor(2.0, dtype=M.torch.float64)),
    ("unit_source", M1, 1, lambda M: M.operator.Laplacian() + M.operator.Convection() + 3 * M.operator.ImplicitSource()),
    ("ks_by_hand", M1, 1, lambda M: -M.operator.Laplacian() - M.operator.Biharmonic() - M.operator.Convection()),
    ("number_minus_operator", M1, 1, lambda M: 2 - M.operator.Laplacian()),
    ("operator_plus_number", M1, 1, lambda M: M.operator.Laplacian() + 1.0),
    ("derivative_sum_2d", M2, 1, lambda M: M.operator.SpatialDerivative(0, 2) - 0.5 * M.operator.SpatialDerivative(1, 1)),
    ("vorticity_2d", M2, 1, lambda M: 1e-2 * M.operator.Laplacian() - M.operator.VorticityConvection()),
    ("conservative_2d", M2, 2, lambda M: M.operator.ConservativeConvection() * 0.5 + M.operator.Laplacian()),
    ("ns_pressure_2d", M2, 2, lambda M: M.operator.NSPressureConvection() - 0.1 * M.operator.Laplacian()),
]


def field(mesh, channels, seed=3):
    rng = np.random.Generator(np.random.PCG64(seed))
    shape = (2, channels) + tuple(n for _, _, n in mesh)
    u = rng.standard_normal(shape)
    # keep the field smooth: drop the upper half of the modes on every axis
    axes = tuple(range(2, u.ndim))
    f = np.fft.fftn(u, axes=axes)
    for ax in axes:
        n = u.shape[ax]
        k = np.abs(np.fft.fftfreq(n, 1.0 / n))
        shape_k = [1] * u.ndim
        shape_k[ax] = n
        f = f * (k <= n // 4).reshape(shape_k)
    return np.fft.ifftn(f, axes=axes).real


def evaluate(M, name, mesh, channels, build):
    """The expression's one-shot value (numpy) or the name of the exception it raised."""
    try:
        op = build(M)
        out = op(u=M.torch.tensor(field(mesh, channels), dtype=M.torch.float64), mesh=mesh)
        return out.detach().numpy()
    except Exception as e:  # noqa: BLE001 -- the error type is part of the recorded behaviour
        return type(e).__name__


def main(ref_root: str) -> None:
    sys.path.insert(0, ref_root)
    sys.path.insert(0, HERE)
    sys.path.insert(0, REPO)
    import cases as C

    M = C.namespace("torchfsm")
    out = {}
    for name, mesh, channels, build in EXPRESSIONS:
        v = evaluate(M, name, mesh, channels, build)
        out[name] = np.array(v) if isinstance(v, str) else v
        print(name, v if isinstance(v, str) else v.shape)
    np.savez(os.path.join(HERE, "algebra_reference.npz"), **out)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TORCHFSM_REFERENCE")
    if not ref:
        sys.exit(f"usage: python {os.path.relpath(__file__)} <reference source tree> (or set TORCHFSM_REFERENCE)")
    main(ref)
