"""bem_solve's outer loop against the reference's own bem_solve
(electrodrive/core/bem.py:1550-2695, fixtures in tests/golden/refine_cases.npz
written by it): h-refinement with best-pass selection, the stop on the
boundary-residual target, and the failure chain (GMRES, a retry without the
preconditioner, damped Jacobi) ending in the reference's error result.

The refinement cases run 10-step GMRES cycles to a 1e-4 tolerance, so every
pass stops at a boundary residual far above rounding and the choice between
passes is reproducible (the reference itself, run twice, reproduces its
residuals to 1e-7 relative)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
K_E = 1.0 / (4.0 * np.pi * 8.854187817e-12)
R = np.load(os.path.join(GOLDEN, "refine_cases.npz"))

SPHERE0 = dict(conductors=[dict(type="sphere", radius=1.0, center=[0.0, 0.0, 0.0], potential=0.0)],
               charges=[dict(type="point", q=1.0, pos=[0.0, 0.0, 2.0])])
SPHERE1 = dict(conductors=[dict(type="sphere", radius=1.0, center=[0.0, 0.0, 0.0], potential=1.0)],
               charges=[dict(type="point", q=1.0, pos=[0.0, 0.0, 2.0])])
TORUS = dict(conductors=[dict(type="torus", major_radius=1.0, minor_radius=0.35, potential=1.0)],
             charges=[dict(type="point", q=1.0, pos=[1.6, 0.3, 0.2])])
CASES = {
    "sphere_stop_on_bc": (SPHERE0, dict(initial_h=0.8, max_refine_passes=3, target_bc_inf_norm=1e-2)),
    "sphere_refine3_v1": (SPHERE1, dict(initial_h=0.8, max_refine_passes=3, target_bc_inf_norm=1e-12,
                                        gmres_restart=10, gmres_tol=1e-4)),
    "torus_refine2_near": (TORUS, dict(initial_h=0.25, max_refine_passes=2, target_bc_inf_norm=1e-12,
                                       use_near_quadrature_matvec=True, gmres_restart=10, gmres_tol=1e-4)),
    "sphere_fallback": (SPHERE0, dict(initial_h=0.8, max_refine_passes=1, gmres_tol=1e-30, gmres_restart=20,
                                      gmres_maxiter=20)),
}


def _cfg(over):
    from electrodrive_gb300.utils.config import BEMConfig

    cfg = BEMConfig(fp64=True)
    for k, v in over.items():
        setattr(cfg, k, v)
    return cfg


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name", ["sphere_stop_on_bc", "sphere_refine3_v1", "torus_refine2_near"])
def test_refinement_loop_matches_reference(cuda_lib, name):
    from electrodrive_gb300.core.bem import bem_solve

    spec, over = CASES[name]
    res = bem_solve(spec, _cfg(over))
    assert "error" not in res, res.get("error")
    ref_passes = R[f"{name}__passes"]
    hist = res["refinement_history"]
    assert len(hist) == ref_passes.shape[0]
    for p, rp in zip(hist, ref_passes):
        assert p["pass"] == int(rp[0]) and p["h"] == pytest.approx(rp[1], rel=1e-12) and p["dof"] == int(rp[2])
        assert p["gmres_info"]["code"] == int(rp[6])
        if over.get("gmres_tol"):
            # residuals and energies far above rounding: compare them
            assert p["gmres_info"]["iters"] == int(rp[5])
            assert p["bc_resid_linf"] == pytest.approx(rp[3], rel=1e-4)
            assert p["energy_A"] == pytest.approx(rp[4], rel=1e-5)
    best = R[f"{name}__best"]
    ms = res["mesh_stats"]
    assert ms["n_panels"] == int(best[0]) and ms["h_final"] == pytest.approx(best[1], rel=1e-12)
    sigma = res["surface_charge_density"]
    assert isinstance(sigma, np.ndarray) and sigma.shape == R[f"{name}__sigma"].shape
    assert _rel(sigma, R[f"{name}__sigma"]) < 1e-5
    assert np.allclose(res["sample_points"], R[f"{name}__sample_points"], rtol=0, atol=1e-12)
    # boundary samples V_free + A sigma: a grounded case sits at rounding level
    # of the ~K_E free-space potential (1e-4 here), so the tolerance carries
    # a term of that size beside the relative one
    bs = R[f"{name}__boundary_samples"]
    tol = 1e-4 * np.max(np.abs(bs)) + 1e-12 * K_E
    assert np.max(np.abs(np.asarray(res["boundary_samples"]) - bs)) <= tol


def test_failed_solve_falls_back_and_reports_the_reference_error(cuda_lib):
    from electrodrive_gb300.core.bem import bem_solve

    spec, over = CASES["sphere_fallback"]
    res = bem_solve(spec, _cfg(over))
    ref = str(R["sphere_fallback__error"])
    assert "error" in res
    # same chain: preconditioned GMRES (code 1), the retry without it, then
    # damped Jacobi diverging to a non-finite residual
    assert res["error"].startswith("BEM linear solve failed: GMRES(code=1,") and ref.startswith(
        "BEM linear solve failed: GMRES(code=1,")
    assert res["error"].endswith("Jacobi(resid=inf)") and ref.endswith("Jacobi(resid=inf)")
    assert res["jacobi_resid"] == float("inf")
