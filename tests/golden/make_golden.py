"""Generate the golden vectors under tests/golden/ by running the reference.

Run in a container where the reference (torchfsm 0.0.4) is importable:

    python tests/golden/make_golden.py <reference source tree>

The reference is imported from the given source tree and run on the CPU in
float64 for every case of ``cases.py`` (``CASES`` and ``CALLBACK_CASES``); the
initial condition, the final physical state and (where recorded) the physical
trajectory are stored in ``<case>.npz``. ``phi_coefs.npz`` holds the reference's SETDRK4 / ETDRK
coefficient tables for a few linear symbols and ``masks.npz`` its 2/3 dealias
masks. These files are the pins of the numpy oracle and of the GPU path; the
GPU tests never read the reference itself.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def main(ref_root: str) -> None:
    sys.path.insert(0, ref_root)
    sys.path.insert(0, REPO)
    import torch

    torch.set_num_threads(max(1, os.cpu_count() or 1))
    import torchfsm  # noqa: F401  (the reference)
    from torchfsm.mesh import FourierMesh
    from torchfsm.traj_recorder import AutoRecorder
    from torchfsm.integrator._stable_etdrk._uncached import UnCachedSETDRK4, UnCachedSETDRK3
    from torchfsm.integrator._etdrk import ETDRK2

    sys.path.insert(0, HERE)
    import cases as C

    M = C.namespace("torchfsm")
    only = set(sys.argv[2:])
    for name, case in list(C.CASES.items()) + list(C.CALLBACK_CASES.items()):
        if only and name not in only:
            continue
        u0 = C.initial_condition(name)
        op = case["build"](M)
        if case.get("integrator"):
            C.set_case_integrator(op, M, case["integrator"])
        rec_fn = C.record_fn(name)
        rec = AutoRecorder(control_func=rec_fn) if rec_fn is not None else None
        out = op.integrate(
            u_0=torch.tensor(u0, dtype=torch.float64),
            mesh=case["mesh"],
            dt=case["dt"],
            step=case["step"],
            trajectory_recorder=rec,
        )
        # Large arrays are stored in float32 (6e-8 relative, far inside the 1e-5 parity bar)
        # and large initial conditions not at all (they are regenerated from their seed).
        def small(x):
            return x if x.size <= 131072 else x.astype(np.float32)

        payload = {"u0": u0} if u0.size <= 65536 else {}
        if rec is not None:
            payload["traj"] = small(out.numpy())
            payload["final"] = small(out[:, -1].numpy())
        else:
            payload["final"] = small(out.numpy())
        payload["integrator"] = np.array(type(op._state_dict["integrator"]).__name__)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **payload)
        print(name, payload["final"].shape, payload["integrator"])

    # Large batches at the benchmarked kernel instances: the kept samples' final fields and every
    # sample's L2 norm.
    for name, case in C.LARGE_CASES.items():
        if only and name not in only:
            continue
        u0 = C.initial_condition(name)
        op = case["build"](M)
        out = op.integrate(u_0=torch.tensor(u0, dtype=torch.float64), mesh=case["mesh"], dt=case["dt"],
                           step=case["step"]).numpy()
        keep = np.asarray(case["keep"], dtype=np.int64)
        kept = out[keep]
        norms = np.sqrt((out.reshape(out.shape[0], -1) ** 2).sum(axis=1))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), keep=keep,
                            final_kept=kept if kept.size <= 131072 else kept.astype(np.float32), norms=norms,
                            integrator=np.array(type(op._state_dict["integrator"]).__name__))
        print(name, kept.shape, "norms", norms.min(), norms.max())

    # One-shot evaluation (Operator.__call__, solve, functional.*) in float64.
    for name, case in C.APPLY_CASES.items():
        if only and name not in only:
            continue
        u = torch.tensor(C.apply_input(name), dtype=torch.float64)
        out = case["fn"](M, u, case["mesh"])
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), out=out.numpy())
        print(name, tuple(out.shape))

    # Gradients by the reference's own autograd (float64): d loss / d u0, d loss / d nu.
    for name, case in C.GRAD_CASES.items():
        if only and name not in only:
            continue
        u0 = torch.tensor(C.grad_initial_condition(name), dtype=torch.float64)
        with torch.no_grad():
            target = M.pde.Burgers(case["nu_target"]).integrate(u_0=u0, mesh=case["mesh"], dt=case["dt"],
                                                                 step=case["step"])
        nu = torch.tensor(case["nu"], dtype=torch.float64, requires_grad=True)
        x = u0.clone().requires_grad_(True)
        op = nu * M.operator.Laplacian() - M.operator.Convection()
        out = op.integrate(u_0=x, mesh=case["mesh"], dt=case["dt"], step=case["step"])
        loss = ((out - target) ** 2).mean()
        loss.backward()
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), u0=u0.numpy(), target=target.numpy(),
                            loss=np.array(loss.item()), grad_u0=x.grad.numpy(), grad_nu=np.array(nu.grad.item()))
        print(name, "loss", loss.item(), "grad_nu", nu.grad.item())

    # Gradients of the other differentiable programs by the reference's autograd (float64).
    for name, case in C.GENERIC_GRAD_CASES.items():
        if only and name not in only:
            continue
        u0 = torch.tensor(C.generic_grad_initial_condition(name), dtype=torch.float64)
        with torch.no_grad():
            target = C.build_generic_grad_op(name, M, case["coef_target"]).integrate(
                u_0=u0, mesh=case["mesh"], dt=case["dt"], step=case["step"])
        c = torch.tensor(case["coef"], dtype=torch.float64, requires_grad=True)
        x = u0.clone().requires_grad_(True)
        out = C.build_generic_grad_op(name, M, c).integrate(u_0=x, mesh=case["mesh"], dt=case["dt"], step=case["step"])
        loss = ((out - target) ** 2).mean()
        loss.backward()
        # the FP32 floor: the reference's own float32 autograd on the same inputs, against its float64
        # gradient (stiff symbols such as KdV's i k^3 amplify the rounding of every step)
        c32 = torch.tensor(case["coef"], dtype=torch.float32, requires_grad=True)
        x32 = u0.float().requires_grad_(True)
        out32 = C.build_generic_grad_op(name, M, c32).integrate(u_0=x32, mesh=case["mesh"], dt=case["dt"],
                                                                 step=case["step"])
        ((out32 - target.float()) ** 2).mean().backward()
        fp32_u = float(torch.linalg.vector_norm(x32.grad.double() - x.grad) / torch.linalg.vector_norm(x.grad))
        grad_coef, coef_source = c.grad.item(), "autograd"
        if not np.isfinite(grad_coef):
            # ETDRK1/2: the reference's coefficient tables choose the L == 0 limit with torch.where, and the
            # gradient of the branch not taken (0/0 at the k = 0 mode) makes its autograd NaN; the
            # reference's float64 loss differentiated by central differences stands in for it
            eps = 1e-6 * max(1.0, abs(case["coef"]))

            def loss_at(cv):
                with torch.no_grad():
                    o = C.build_generic_grad_op(name, M, cv).integrate(u_0=u0, mesh=case["mesh"], dt=case["dt"],
                                                                       step=case["step"])
                return float(((o - target) ** 2).mean())

            grad_coef = (loss_at(case["coef"] + eps) - loss_at(case["coef"] - eps)) / (2 * eps)
            coef_source = "central differences of the float64 loss (the reference's autograd gives NaN)"
        fp32_c = abs(c32.grad.item() - grad_coef) / abs(grad_coef)  # NaN where the float32 autograd is NaN
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), u0=u0.numpy(), target=target.numpy(),
                            loss=np.array(loss.item()), grad_u0=x.grad.numpy(), grad_coef=np.array(grad_coef),
                            grad_coef_source=np.array(coef_source),
                            fp32_grad_u0_rel_l2=np.array(fp32_u), fp32_grad_coef_rel=np.array(fp32_c))
        print(name, "loss", loss.item(), "grad_coef", grad_coef, coef_source, "fp32 floor", fp32_u, fp32_c)

    if only:
        return
    # Coefficient tables (integrator/_stable_etdrk/_uncached.py:180-211, _etdrk.py:54-82).
    tabs = {}
    for tag, mesh_info, lin_fn, dt in (
        ("ks1d", [(0, 32 * np.pi, 64)], lambda fm: -fm.laplacian() - fm.laplacian() ** 2, 0.1),
        ("ns2d", [(0, 2 * np.pi, 32)] * 2, lambda fm: 1e-3 * fm.laplacian(), 1e-3),
        ("kdv1d", [(0, 20.0, 64)], lambda fm: -fm.grad(0, 3), 1e-3),
    ):
        fm = FourierMesh(mesh_info, dtype=torch.float64)
        L = lin_fn(fm)
        tabs[f"{tag}_L"] = L.numpy()
        for M_, r_ in ((16, 1.0), (32, 2.0)):
            it = UnCachedSETDRK4(dt, L, None, M_, r_)
            key = f"{tag}_m{M_}"
            tabs[f"{key}_E"] = it._exp_term.numpy()
            tabs[f"{key}_E2"] = it._half_exp_term.numpy()
            for i in (1, 4, 5, 6):
                tabs[f"{key}_c{i}"] = getattr(it, f"_coef_{i}").numpy()
        it3 = UnCachedSETDRK3(dt, L, None, 16, 1.0)
        for i in (1, 2, 3, 4, 5):
            tabs[f"{tag}_s3_c{i}"] = getattr(it3, f"_coef_{i}").numpy()
        e2 = ETDRK2(dt, L, None)
        tabs[f"{tag}_e2_c1"] = e2._coef_1.numpy()
        tabs[f"{tag}_e2_c2"] = e2._coef_2.numpy()
        tabs[f"{tag}_dt"] = np.array(dt)
    np.savez_compressed(os.path.join(HERE, "phi_coefs.npz"), **tabs)

    # Dealias masks (mesh.py:443-461).
    masks = {}
    for n in (12, 16, 48, 96, 128, 256):
        for dt_name, dtype in (("f32", torch.float32), ("f64", torch.float64)):
            for rate in (2.0 / 3.0, 0.5, 1.0):
                fm = FourierMesh([(0, 2 * np.pi, n)], dtype=dtype)
                fm.set_default_rel_freq_threshold(rate)
                masks[f"n{n}_{dt_name}_r{rate:.4f}"] = fm.low_pass_filter(rate).numpy().reshape(-1)
    np.savez_compressed(os.path.join(HERE, "masks.npz"), **masks)
    print("phi_coefs, masks written")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TORCHFSM_REFERENCE")
    if not ref:
        sys.exit(f"usage: python {os.path.relpath(__file__)} <reference source tree> (or set TORCHFSM_REFERENCE)")
    main(ref)
