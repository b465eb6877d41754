"""GPU FMM matvec parity.

* P2P against the reference's own P2P potentials (fixture) and the oracle;
* the full operator against the oracle's FP64 FMM on the same tree and lists
  (same algorithm: only FP32 rounding separates them) and against FP64
  direct summation (the binding accuracy check: 1e-5 relative at p = 8);
* against the reference FMM's potentials within the reference's own error
  budget: ||V - V_ref|| <= ||V_ref - V_dense|| + 1e-5 ||V_dense||.
Tolerances: FP32 paths 1e-5 relative L2 (2e-6 vs the same-algorithm oracle);
FP64 paths 1e-10.
"""
import glob
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

K_E = 1.0 / (4.0 * np.pi * 8.854187817e-12)


def _plan(pts, leaf=64, theta=0.5, p=8, max_depth=32):
    from electrodrive_gb300 import _lib

    return _lib.Plan(torch.as_tensor(pts).cuda(), leaf_size=leaf, max_depth=max_depth, mac_theta=theta,
                     expansion_order=p)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "tree_*.npz"))),
                         ids=lambda p: os.path.basename(p)[5:-4])
def test_p2p_matches_reference_potentials(cuda_lib, path):
    z = np.load(path)
    plan = _plan(z["points"], int(z["leaf_size"]), float(z["theta"]), max_depth=int(z["max_depth"]))
    plan.set_charges(torch.as_tensor(z["charges"]).cuda())
    phi = plan.p2p().cpu().numpy()
    ref = z["p2p_potential_tree"].astype(np.float64)
    tol = 1e-12 if z["points"].dtype == np.float64 else 2e-6
    assert rel(phi, ref) < tol


@pytest.mark.parametrize("n,p", [(5000, 8), (20000, 8), (8000, 4), (6000, 6), (4000, 10), (3000, 1), (7000, 7),
                                 (5000, 5), (3000, 2), (4000, 3)])
def test_matvec_matches_oracle_fmm_fp32(cuda_lib, oracle, n, p):
    rng = np.random.default_rng(n + p)
    pts = rng.random((n, 3)).astype(np.float32)
    sigma = rng.uniform(-1, 1, n).astype(np.float32)
    areas = rng.uniform(0.5, 1.5, n).astype(np.float32) / n
    plan = _plan(pts, 64, 0.5, p)
    v = plan.matvec(torch.as_tensor(sigma).cuda(), torch.as_tensor(areas).cuda(), None, k_e=1.0).cpu().numpy()
    t = oracle.build_tree(pts, 64, 32)
    lists = oracle.build_lists(t, 0.5)
    ref = oracle.fmm_matvec(t, lists, pts, sigma, areas, None, p=p, ke=1.0)
    assert rel(v, ref) < 2e-6
    if p == 8:
        d = oracle.direct(pts, sigma.astype(np.float64) * areas)
        assert rel(v, d) < 1e-5


def _torus_points(n_u, n_v):
    u = np.linspace(0, 2 * np.pi, n_u, endpoint=False)[:, None]
    v = np.linspace(0, 2 * np.pi, n_v, endpoint=False)[None, :]
    x = (1.0 + 0.35 * np.cos(v)) * np.cos(u)
    y = (1.0 + 0.35 * np.cos(v)) * np.sin(u)
    z = 0.35 * np.sin(v) + 0 * u
    return np.stack([x, y, z], -1).reshape(-1, 3)


@pytest.mark.parametrize("p", [3, 6, 7, 8])
@pytest.mark.parametrize("kind", ["cube", "torus"])
def test_matvec_fp64_plan_matches_oracle(cuda_lib, oracle, p, kind):
    rng = np.random.default_rng(11 + p)
    pts = rng.random((6000, 3)) if kind == "cube" else _torus_points(120, 50)
    n = pts.shape[0]
    sigma = rng.uniform(-1, 1, n)
    areas = rng.uniform(0.5, 1.5, n) / n
    si = rng.uniform(0, 1e3, n)
    plan = _plan(pts, 48, 0.5, p)
    v = plan.matvec(torch.as_tensor(sigma).cuda(), torch.as_tensor(areas).cuda(), torch.as_tensor(si).cuda(),
                    k_e=K_E).cpu().numpy()
    t = oracle.build_tree(pts, 48, 32)
    lists = oracle.build_lists(t, 0.5)
    ref = oracle.fmm_matvec(t, lists, pts, sigma, areas, si, p=p)
    assert rel(v, ref) < 1e-10


def test_matvec_fp32_surface_matches_oracle(cuda_lib, oracle):
    """A torus surface grid: its tree has single-point nodes (radius 0),
    which exercise the parent-relative expansion scale."""
    rng = np.random.default_rng(5)
    pts = _torus_points(200, 80).astype(np.float32)
    n = pts.shape[0]
    sigma = rng.uniform(-1, 1, n).astype(np.float32)
    areas = np.full(n, 1.0 / n, np.float32)
    plan = _plan(pts, 64, 0.5, 8)
    v = plan.matvec(torch.as_tensor(sigma).cuda(), torch.as_tensor(areas).cuda(), None, k_e=1.0).cpu().numpy()
    t = oracle.build_tree(pts, 64, 32)
    lists = oracle.build_lists(t, 0.5)
    ref = oracle.fmm_matvec(t, lists, pts, sigma, areas, None, p=8, ke=1.0)
    assert rel(v, ref) < 2e-6
    assert rel(v, oracle.direct(pts, sigma.astype(np.float64) * areas)) < 1e-5


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "fmm_*.npz"))),
                         ids=lambda p: os.path.basename(p)[4:-4])
def test_public_matvec_against_reference_fmm_and_dense(cuda_lib, path):
    from electrodrive_gb300.fmm3d import make_laplace_fmm_backend

    z = np.load(path)
    c = torch.as_tensor(z["points"])
    a = torch.as_tensor(z["areas"])
    s = torch.as_tensor(z["sigma"])
    si = torch.as_tensor(z["self_integrals"])
    fmm = make_laplace_fmm_backend(c, a, max_leaf_size=int(z["leaf_size"]), theta=float(z["theta"]),
                                   expansion_order=int(z["p"]))
    dense = z["v_dense_reference"].astype(np.float64)
    ref_fmm = z["v_fmm_reference"].astype(np.float64)
    budget = np.linalg.norm(ref_fmm - dense) / np.linalg.norm(dense)
    for sig, sint in ((s, si), (s.cuda(), si.cuda())):
        v = fmm.matvec(sigma=sig, src_centroids=c, areas=a, tile_size=1024, self_integrals=sint)
        assert v.device == sig.device
        v = v.cpu().numpy()
        assert rel(v, dense) < 1e-5
        assert np.linalg.norm(v - ref_fmm) / np.linalg.norm(dense) <= budget + 1e-5


def test_reference_pair_order_switch(cuda_lib, oracle):
    rng = np.random.default_rng(21)
    n = 12000
    pts = np.concatenate([rng.normal(0.3, 0.05, (n // 2, 3)), rng.random((n // 2, 3))]).astype(np.float32)
    sigma = rng.uniform(-1, 1, n).astype(np.float32)
    areas = np.full(n, 1.0 / n, np.float32)
    from electrodrive_gb300 import _lib

    plan = _plan(pts, 32, 0.5, 8)
    v = plan.matvec(torch.as_tensor(sigma).cuda(), torch.as_tensor(areas).cuda(), None, k_e=1.0,
                    flags=_lib.EDFMM_REFERENCE_PAIR_ORDER).cpu().numpy()
    t = oracle.build_tree(pts, 32, 32)
    lists = oracle.build_lists(t, 0.5)
    ref = oracle.fmm_matvec(t, lists, pts, sigma, areas, None, p=8, ke=1.0, reference_pair_order=True)
    assert rel(v, ref) < 2e-6


def test_stages_compose_to_matvec(cuda_lib):
    from electrodrive_gb300 import _lib

    rng = np.random.default_rng(4)
    n = 9000
    pts = rng.random((n, 3)).astype(np.float32)
    q = torch.as_tensor(rng.uniform(-1, 1, n).astype(np.float32)).cuda()
    ones = torch.ones(n, device="cuda")
    plan = _plan(pts)
    full = plan.matvec(q, ones, None, k_e=1.0)
    plan.set_charges(q)
    for st in ("p2m", "m2m"):
        plan.stage(st)
    plan.stage("m2l", 0)
    plan.stage("l2l")
    far = plan.l2p()
    near = plan.p2p()
    soa = plan.export_tree()
    total = torch.empty_like(full)
    total[soa["index_map"]] = far + near
    assert rel(total.cpu().numpy(), full.cpu().double().numpy()) < 1e-6
    nf = plan.matvec(q, ones, None, k_e=1.0, flags=_lib.EDFMM_NO_FARFIELD)
    assert rel(nf.cpu().numpy(), near[torch.argsort(soa["index_map"])].cpu().double().numpy()) < 1e-6


def test_nonfinite_outputs_are_zeroed(cuda_lib):
    n = 2000
    rng = np.random.default_rng(8)
    pts = rng.random((n, 3)).astype(np.float32)
    plan = _plan(pts)
    sigma = torch.ones(n, device="cuda")
    si = torch.zeros(n, device="cuda")
    si[5] = float("inf")
    v = plan.matvec(sigma, torch.ones(n, device="cuda"), si, k_e=1.0)
    assert v[5].item() == 0.0 and torch.isfinite(v).all()


def test_coincident_points_follow_reference_eps_rule(cuda_lib, oracle):
    """Distinct coincident points in one leaf contribute q / eps, the diagonal 0."""
    pts = np.repeat(np.array([[0.5, 0.5, 0.5], [0.1, 0.2, 0.3]], np.float32), 3, axis=0)
    q = np.array([1, 2, 3, 4, 5, 6], np.float32)
    plan = _plan(pts, 64)
    plan.set_charges(torch.as_tensor(q).cuda())
    phi = plan.p2p().cpu().numpy()
    t = oracle.build_tree(pts, 64, 32)
    lists = oracle.build_lists(t, 0.5)
    ref = oracle.p2p(t.points_tree, q[t.index_map], t.node_ranges, lists.p2p_pairs, float(np.finfo(np.float32).eps))
    assert rel(phi, ref) < 1e-6


@pytest.mark.slow
def test_million_point_matvec_properties(cuda_lib, oracle):
    """The benchmark workload: lists bit-exact, 4,096 sampled targets vs FP64 direct sum."""
    n = 1 << 20
    g = torch.Generator().manual_seed(0)
    pts = torch.rand(n, 3, generator=g, dtype=torch.float64).float()
    q = (2 * torch.rand(n, generator=torch.Generator().manual_seed(1), dtype=torch.float64) - 1).float()
    plan = _plan(pts.numpy(), 64, 0.5, 8)
    v = plan.matvec(q.cuda(), torch.ones(n, device="cuda"), None, k_e=1.0).cpu().numpy()
    t = oracle.build_tree(pts.numpy(), 64, 32)
    lists = oracle.build_lists(t, 0.5)
    p2p, m2l = plan.export_lists()
    assert np.array_equal(m2l.cpu().numpy(), lists.m2l_pairs)
    idx = torch.randperm(n, generator=torch.Generator().manual_seed(3))[:4096].numpy()
    d = oracle.direct(pts.numpy(), q.double().numpy(), idx)
    assert rel(v[idx], d) < 1e-5
