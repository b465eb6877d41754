"""Two-float arithmetic of the FP64 operator (edfmm_plan_set_arithmetic):
M2L and the near field of an FP64 plan evaluated on the FP32 pipe as sums
of two floats.  The matvec stays within 1e-11 of the oracle's FP64 FMM on
the same tree and of the plan's IEEE FP64 matvec, on uniform, clustered,
coincident and surface point sets, with and without the reference's
swapped M2L pair order; a mixed solve whose stopping test uses it meets its
tolerance on the IEEE FP64 operator too."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _points(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "uniform":
        return rng.random((n, 3))
    if kind == "clusters":
        a = 0.02 * rng.normal(size=(n // 2, 3)) + 0.25
        b = 0.05 * rng.normal(size=(n // 3, 3)) + np.array([0.8, 0.7, 0.3])
        return np.concatenate([a, b, rng.random((n - a.shape[0] - b.shape[0], 3))])
    if kind == "coincident":
        p = rng.random((n // 4, 3))
        return np.concatenate([p, p, p, rng.random((n - 3 * (n // 4), 3))])
    from electrodrive_gb300.core.bem_mesh import torus_mesh

    return torus_mesh(1.0, 0.35, 120, 48).centroids


@pytest.mark.parametrize("kind,n", [("uniform", 20000), ("clusters", 15000), ("coincident", 8000), ("torus", 0)])
def test_two_float_matvec_matches_fp64_and_oracle(cuda_lib, oracle, kind, n):
    from electrodrive_gb300._lib import Plan

    pts = _points(kind, n, 3)
    n = pts.shape[0]
    rng = np.random.default_rng(4)
    sigma = rng.uniform(-1, 1, n)
    areas = rng.uniform(0.5, 1.5, n) / n
    T = lambda x: torch.as_tensor(x, dtype=torch.float64, device="cuda")
    plan = Plan(T(pts), leaf_size=64, expansion_order=8)
    v64 = plan.matvec(T(sigma), T(areas), None, k_e=1.0).cpu().numpy()
    plan.set_arithmetic("two_float")
    v2 = plan.matvec(T(sigma), T(areas), None, k_e=1.0).cpu().numpy()
    # the stages alone (far field, then near field) in both modes
    far2 = plan.matvec(T(sigma), T(areas), None, k_e=1.0, flags=4).cpu().numpy()
    near2 = plan.matvec(T(sigma), T(areas), None, k_e=1.0, flags=2).cpu().numpy()
    plan.set_arithmetic("native")
    far64 = plan.matvec(T(sigma), T(areas), None, k_e=1.0, flags=4).cpu().numpy()
    near64 = plan.matvec(T(sigma), T(areas), None, k_e=1.0, flags=2).cpu().numpy()
    scale = np.linalg.norm(v64)
    assert np.linalg.norm(v2 - v64) <= 1e-11 * scale
    assert np.linalg.norm(far2 - far64) <= 1e-11 * scale
    assert np.linalg.norm(near2 - near64) <= 1e-11 * scale
    t = oracle.build_tree(pts, 64, 32)
    lists = oracle.build_lists(t, 0.5)
    ref = oracle.fmm_matvec(t, lists, pts, sigma, areas, None, p=8, ke=1.0)
    assert np.linalg.norm(v2 - ref) <= 1e-11 * np.linalg.norm(ref)


@pytest.mark.parametrize("order,block", [(6, 128), (7, 128), (8, 128), (8, 256)])
def test_packed_and_scalar_two_float_m2l_are_bit_identical(cuda_lib, order, block):
    """The two-float M2L with its rotation matrices on packed FP32x2
    instructions (the default) and in scalar form give the same bits."""
    from electrodrive_gb300._lib import Plan

    pts = _points("clusters", 9000, 7)
    n = pts.shape[0]
    rng = np.random.default_rng(8)
    T = lambda x: torch.as_tensor(x, dtype=torch.float64, device="cuda")
    s, a = T(rng.uniform(-1, 1, n)), T(rng.uniform(0.5, 1.5, n) / n)
    plan = Plan(T(pts), leaf_size=32, expansion_order=order)
    plan.set_arithmetic("two_float")
    plan.set_launch(m2l_tf_block=block)
    out = {}
    for packed in (1, 0):
        plan.set_launch(m2l_packed=packed)
        out[packed] = plan.matvec(s, a, None, k_e=1.0, flags=4)  # far field alone
    assert torch.equal(out[0], out[1])


def test_two_float_reference_pair_order_and_mode_switch(cuda_lib):
    from electrodrive_gb300._lib import EDFMM_REFERENCE_PAIR_ORDER, Plan

    pts = _points("clusters", 12000, 5)
    n = pts.shape[0]
    rng = np.random.default_rng(6)
    T = lambda x: torch.as_tensor(x, dtype=torch.float64, device="cuda")
    s, a = T(rng.uniform(-1, 1, n)), T(np.full(n, 1.0 / n))
    plan = Plan(T(pts), leaf_size=32, expansion_order=8)
    ref = plan.matvec(s, a, None, k_e=1.0, flags=EDFMM_REFERENCE_PAIR_ORDER).cpu().numpy()
    plan.set_arithmetic("two_float")
    got = plan.matvec(s, a, None, k_e=1.0, flags=EDFMM_REFERENCE_PAIR_ORDER).cpu().numpy()
    assert np.linalg.norm(got - ref) <= 1e-11 * np.linalg.norm(ref)
    # FP32 plans accept only native arithmetic
    p32 = Plan(T(pts).float(), leaf_size=32, expansion_order=8)
    with pytest.raises(Exception):
        p32.set_arithmetic("two_float")


def test_mixed_solve_with_two_float_stopping_test(cuda_lib):
    """The FP64 residuals of the refinement (and its stopping test) from the
    two-float operator: the final density meets the 1e-6 tolerance against
    the IEEE FP64 operator as well."""
    from electrodrive_gb300.core.bem import assemble_system, solve_mixed
    from electrodrive_gb300.core.bem_mesh import torus_mesh

    spec = dict(conductors=[dict(type="torus", major_radius=1.0, minor_radius=0.35, potential=1.0)],
                charges=[dict(type="point", q=1.0, pos=[1.6, 0.3, 0.2])])
    S = assemble_system(torus_mesh(1.0, 0.35, 80, 32), spec, kind="fmm", dtypes=(torch.float64, torch.float32),
                        near=True)
    op64, op32, b = S["ops"][torch.float64], S["ops"][torch.float32], S["b"]
    op64.base.plan.set_arithmetic("two_float")
    x, info = solve_mixed(op64, op32, b, A_diag=S["diag"], x0=S["x0"], rtol=1e-6)
    assert info["code"] == 0
    op64.base.plan.set_arithmetic("native")
    rel = float(torch.linalg.norm(b - op64(x)) / torch.linalg.norm(b))
    assert rel <= 1e-6 * (1 + 1e-6)
