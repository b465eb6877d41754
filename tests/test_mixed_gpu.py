"""Mixed FP32/FP64 refinement (core.bem.solve_mixed) on a torus with the near
correction: the solve stops only on an FP64 true residual <= rtol, whether
the first residual of the start comes from the FP32 or the FP64 operator,
and its density matches the plain FP64 GMRES solve of the same system.
"""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torus_system(cuda_lib):
    from electrodrive_gb300.core.bem import assemble_system
    from electrodrive_gb300.core.bem_mesh import torus_mesh

    spec = dict(conductors=[dict(type="torus", major_radius=1.0, minor_radius=0.35, potential=1.0)],
                charges=[dict(type="point", q=1.0, pos=[1.6, 0.3, 0.2])])
    mesh = torus_mesh(1.0, 0.35, 80, 32)
    return assemble_system(mesh, spec, kind="fmm", dtypes=(torch.float64, torch.float32), near=True)


@pytest.mark.parametrize("first", ["fp32", "fp64"])
def test_mixed_solve_stops_on_fp64_residual(torus_system, first):
    from electrodrive_gb300.core.bem import solve_mixed
    from electrodrive_gb300.core.bem_solver import gmres_restart

    S = torus_system
    op64, op32 = S["ops"][torch.float64], S["ops"][torch.float32]
    b = S["b"]
    x, info = solve_mixed(op64, op32, b, A_diag=S["diag"], x0=S["x0"], rtol=1e-6, first_residual=first)
    assert info["code"] == 0, info
    rel = float(torch.linalg.norm(b - op64(x)) / torch.linalg.norm(b))
    assert rel <= 1e-6 * (1 + 1e-9)
    assert abs(rel - info["rel_resid"]) <= 1e-3 * rel  # the reported residual is the FP64 one
    bn = float(torch.linalg.norm(b))
    r0 = float(torch.linalg.norm(b - op64(S["x0"])))
    xp, pinfo = gmres_restart(op64, b, restart=256, tol=1e-9 * bn / r0, maxiter=2000, precond="jacobi",
                              A_diag=S["diag"], x0=S["x0"], early_exit=8)
    assert pinfo["code"] == 0
    # a 1e-6 residual leaves sigma about 1e-4 from the converged density on
    # this system (the same holds for plain FP64 GMRES stopped there); the
    # refinement run to 1e-7 brings it within 1e-5
    assert float(torch.linalg.norm(x - xp) / torch.linalg.norm(xp)) < 1e-4
    x7, info7 = solve_mixed(op64, op32, b, A_diag=S["diag"], x0=S["x0"], rtol=1e-7, first_residual=first)
    assert info7["code"] == 0
    assert float(torch.linalg.norm(b - op64(x7)) / torch.linalg.norm(b)) <= 1e-7 * (1 + 1e-9)
    assert float(torch.linalg.norm(x7 - xp) / torch.linalg.norm(xp)) < 1e-5
    if first == "fp32":
        # the start's residual came from the FP32 operator: one FP64 application per refinement step
        assert info["matvec64"] == info["outer"]
    else:
        assert info["matvec64"] == info["outer"] + 1


def test_autotuned_inner_operator_meets_its_bound_and_the_solve_converges(torus_system):
    from electrodrive_gb300.core.bem import autotune_inner_operator, solve_mixed

    S = torus_system
    op64 = S["ops"][torch.float64]
    op32, trials = autotune_inner_operator(op64, S["centroids"], S["areas"], S["self_corr"],
                                           near=S["ops"][torch.float32].near, orders=(8, 6), max_rel_error=3e-7,
                                           use_cache=False)
    assert {t["expansion_order"] for t in trials} == {8, 6}
    assert {t["launch"]["near_overlap"] for t in trials} == {0, 1}
    launch = op32.base.plan.get_launch()
    chosen = [t for t in trials if t["expansion_order"] == op32.base.plan.info.expansion_order
              and t["launch"]["near_overlap"] == launch["near_overlap"]][0]
    from electrodrive_gb300.fmm3d.autotune import TIME_SLACK, select_trial

    assert chosen["rel_error"] <= 3e-7
    assert chosen is select_trial(trials, 3e-7)  # the most accurate of those within 5% of the fastest
    assert chosen["ms"] <= (1 + TIME_SLACK) * min(t["ms"] for t in trials if t["rel_error"] <= 3e-7)
    b = S["b"]
    x, info = solve_mixed(op64, op32, b, A_diag=S["diag"], x0=S["x0"], rtol=1e-6)
    assert info["code"] == 0
    assert float(torch.linalg.norm(b - op64(x)) / torch.linalg.norm(b)) <= 1e-6 * (1 + 1e-9)
