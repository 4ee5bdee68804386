"""The numpy FP64 oracle against golden vectors produced by the reference itself."""

import os

import numpy as np
import pytest

import cases as C
from oracle import spectral as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


@pytest.mark.parametrize("name", sorted(C.CASES))
def test_oracle_matches_reference(name):
    case = C.CASES[name]
    g = _load(name)
    u0 = C.initial_condition(name)
    if "u0" in g:
        np.testing.assert_array_equal(u0, g["u0"])  # the seeded generator is reproducible
    # float64 fixtures pin the oracle to 1e-10; large fixtures are stored in float32
    def tol(x):
        return 1e-10 if x.dtype == np.float64 else 1e-6

    lin, nl = C.oracle_terms(name)
    final, traj = S.integrate(
        u0, case["mesh"], lin, nl, case["dt"], case["step"],
        integrator=case.get("integrator", "auto"), record=C.record_fn(name),
    )
    assert S.rel_l2(final, g["final"]) < tol(g["final"])
    if "traj" in g:
        assert traj.shape == g["traj"].shape
        assert S.rel_l2(traj, g["traj"]) < tol(g["traj"])


@pytest.mark.parametrize("name", sorted(C.LARGE_CASES))
def test_oracle_matches_reference_large(name):
    """The oracle on the samples of a large case that it integrates alone, against the reference's
    fields of the same samples (stored in float32 above 131072 values)."""
    case = C.LARGE_CASES[name]
    g = _load(name)
    keep = list(g["keep"])
    u0 = C.initial_condition(name)
    lin, nl = C.oracle_terms(name)
    for b in case["oracle_samples"]:
        final, _ = S.integrate(u0[b:b + 1], case["mesh"], lin, nl, case["dt"], case["step"])
        ref = g["final_kept"][keep.index(b)]
        tol = 1e-10 if ref.dtype == np.float64 else 1e-6
        assert S.rel_l2(final[0], ref) < tol
        assert abs(np.sqrt((final ** 2).sum()) - g["norms"][b]) < tol * g["norms"][b]


@pytest.mark.parametrize("tag,dt_mesh", [
    ("ks1d", [(0, 32 * np.pi, 64)]),
    ("ns2d", [(0, 2 * np.pi, 32)] * 2),
    ("kdv1d", [(0, 20.0, 64)]),
])
def test_phi_coefficients_match_reference(tag, dt_mesh):
    g = np.load(os.path.join(GOLDEN, "phi_coefs.npz"))
    L = g[f"{tag}_L"]
    dt = float(g[f"{tag}_dt"])
    for m, r in ((16, 1.0), (32, 2.0)):
        tabs = S.setdrk_coefs(4, L, dt, m, r)
        key = f"{tag}_m{m}"
        for name in ("E", "E2", "c1", "c4", "c5", "c6"):
            ref = g[f"{key}_{name}"]
            np.testing.assert_allclose(tabs[name], ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())
    t3 = S.setdrk_coefs(3, L, dt)
    for i in range(1, 6):
        ref = g[f"{tag}_s3_c{i}"]
        np.testing.assert_allclose(t3[f"c{i}"], ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())
    e2 = S.etdrk_coefs(2, L, dt)
    for i in (1, 2):
        ref = g[f"{tag}_e2_c{i}"]
        np.testing.assert_allclose(e2[f"c{i}"], ref, rtol=1e-9, atol=1e-12 * np.abs(ref).max())


def test_masks_match_reference():
    g = np.load(os.path.join(GOLDEN, "masks.npz"))
    for key in g.files:
        n = int(key.split("_")[0][1:])
        dtype = np.float32 if "_f32_" in key else np.float64
        rate = {"0.6667": 2.0 / 3.0, "0.5000": 0.5, "1.0000": 1.0}[key.split("_r")[-1]]
        m = S.OMesh([(0, 2 * np.pi, n)], dtype).low_pass_filter(rate).reshape(-1)
        np.testing.assert_array_equal(m, g[key], err_msg=key)


@pytest.mark.parametrize("name", sorted(n for n, c in C.APPLY_CASES.items() if "lin" in c))
def test_oracle_one_shot_evaluation_matches_reference(name):
    case = C.APPLY_CASES[name]
    out = S.apply_operator(C.apply_input(name), case["mesh"], case["lin"], case["nl"])
    assert S.rel_l2(out, _load(name)["out"]) < 1e-10
