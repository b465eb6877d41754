"""Field at arbitrary targets (bem_E_field_targets, BEMSolution.eval_V_E_batched).

The induced field of panel charges agrees with the reference's own
bem_E_field_targets on its fixtures (tests/golden/make_golden.py, group
"efield"), including a target on a source centroid (the 1e-24 clamp of r^2);
the free-space field of point charges agrees with the reference's
_free_space_E_field_at_points; and the field of a solved sphere is minus the
gradient of its potential.
"""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

Z = np.load(os.path.join(GOLDEN, "efield_cases.npz"))
CASES = sorted({k.split("__")[0] for k in Z.files})
CHARGES = [(1.5, (0.2, 0.3, 1.4)), (-0.5, (0.9, -0.4, 0.1))]


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name", CASES)
def test_free_space_field_matches_reference(name):
    from electrodrive_gb300.core.bem_near import point_charge_field

    t = torch.as_tensor(Z[f"{name}__targets"])
    e = point_charge_field(t, CHARGES).numpy()
    tol = 1e-12 if t.dtype == torch.float64 else 1e-6
    assert _rel(e, Z[f"{name}__E_free"]) < tol


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_induced_field_matches_reference(cuda_lib, name):
    from electrodrive_gb300.core.bem_kernel import bem_E_field_targets

    T = lambda k: torch.as_tensor(Z[f"{name}__{k}"]).cuda()
    e = bem_E_field_targets(T("targets"), T("centroids"), T("areas"), T("sigma")).cpu().numpy()
    ref = Z[f"{name}__E"].astype(np.float64)
    tol = 1e-12 if Z[f"{name}__targets"].dtype == np.float64 else 2e-5
    assert _rel(e, ref) < tol
    # row by row as well: the worst target within the same bound times 10
    worst = max(_rel(e[i], ref[i]) for i in range(ref.shape[0]) if np.linalg.norm(ref[i]) > 0)
    assert worst < 10 * tol


@pytest.mark.gpu
def test_solution_field_is_minus_potential_gradient(cuda_lib):
    from electrodrive_gb300.core.bem import BEMSolution

    rng = np.random.default_rng(3)
    c = torch.as_tensor(rng.normal(size=(3000, 3)), device="cuda")
    c = c / c.norm(dim=1, keepdim=True)
    a = torch.full((3000,), 4 * np.pi / 3000, dtype=torch.float64, device="cuda")
    s = torch.as_tensor(rng.uniform(-1, 1, 3000), device="cuda")
    sol = BEMSolution(centroids=c, areas=a, sigma=s, charges=[(1.0, (0.0, 0.0, 2.5))])
    p = torch.as_tensor(rng.normal(size=(20, 3)), device="cuda")
    p = p / p.norm(dim=1, keepdim=True) * 1.6
    v, e = sol.eval_V_E_batched(p)
    assert v.shape == (20,) and e.shape == (20, 3)
    h = 1e-5
    g = torch.stack([(sol.eval(p + h * d) - sol.eval(p - h * d)) / (2 * h)
                     for d in torch.eye(3, dtype=torch.float64, device="cuda")], dim=1)
    assert float(torch.linalg.norm(e + g) / torch.linalg.norm(e)) < 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_fmm_field_matches_dense_field(cuda_lib, dtype):
    """The FMM field at targets (near sums over the P2P lists, minus the
    gradient of the local expansions) agrees with the dense field to the
    FMM's accuracy at p = 8, for targets inside, around and outside the cloud."""
    from electrodrive_gb300.core.bem_kernel import bem_E_field_targets

    rng = np.random.default_rng(11)
    T = lambda x: torch.as_tensor(x, dtype=dtype, device="cuda")
    c = T(rng.random((20000, 3)))
    a = T(rng.uniform(0.5, 1.5, 20000) / 20000)
    s = T(rng.uniform(-1, 1, 20000))
    x = T(rng.random((3000, 3)) * 1.6 - 0.3)
    ed = bem_E_field_targets(x, c, a, s).double()
    ef = bem_E_field_targets(x, c, a, s, method="fmm").double()
    assert ef.shape == (3000, 3)
    assert float(torch.linalg.norm(ef - ed) / torch.linalg.norm(ed)) < 3e-5
