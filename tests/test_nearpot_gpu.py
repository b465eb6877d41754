"""Target-side near quadrature of the induced potential
(bem_near.near_potential_correction, BEMSolution.eval with near_quadrature).

Against the reference's own _apply_near_quadrature_potentials on its
fixtures (tests/golden/make_golden.py, group "nearpot"): targets close to a
sphere and a torus, on centroids (the r < 1e-12 branch) and far away, each
correction to 1e-10 of its size.
"""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
Z = np.load(os.path.join(GOLDEN, "nearpot_cases.npz"))
CASES = sorted({k.split("__")[0] for k in Z.files})


@pytest.mark.parametrize("name", CASES)
def test_target_near_correction_matches_reference(cuda_lib, name):
    from electrodrive_gb300.core.bem_near import near_potential_correction

    T = lambda k: torch.as_tensor(Z[f"{name}__{k}"]).cuda()
    factor, order, depth = Z[f"{name}__meta"]
    v = near_potential_correction(T("v_in"), T("targets"), T("centroids"), T("areas"), T("sigma"),
                                  T("panel_vertices"), distance_factor=float(factor), quad_order=int(order),
                                  max_depth=int(depth)).cpu().numpy()
    d_ours = v - Z[f"{name}__v_in"]
    d_ref = Z[f"{name}__v_out"] - Z[f"{name}__v_in"]
    assert np.count_nonzero(d_ref) > 10  # the fixture exercises the correction
    err = np.abs(d_ours - d_ref)
    assert np.all(err <= 1e-10 * np.abs(d_ref) + 1e-12 * np.abs(d_ref).max()), err.max()
    far = slice(45, 55)  # targets far from every panel: untouched
    assert np.array_equal(v[far], Z[f"{name}__v_in"][far])


def test_solution_eval_uses_near_quadrature(cuda_lib):
    from electrodrive_gb300.core.bem import BEMSolution

    name = "torus"
    T = lambda k: torch.as_tensor(Z[f"{name}__{k}"]).cuda()
    plain = BEMSolution(centroids=T("centroids"), areas=T("areas"), sigma=T("sigma"))
    near = BEMSolution(centroids=T("centroids"), areas=T("areas"), sigma=T("sigma"), panel_vertices=T("panel_vertices"),
                       near_quadrature=True, near_quad_dist_factor=1.5, near_quad_max_depth=4)
    x = T("targets")[:40]
    v0, v1 = plain.eval(x), near.eval(x)
    from electrodrive_gb300.core.bem_near import near_potential_correction

    ref = near_potential_correction(v0, x, T("centroids"), T("areas"), T("sigma"), T("panel_vertices"),
                                    distance_factor=1.5, quad_order=2, max_depth=4)
    assert torch.equal(v1, ref)
    assert not torch.equal(v0, v1)
