"""GPU octree and interaction lists: bit-exact against the reference's own
fixtures and against the oracle at sizes the fixtures do not reach."""
import glob
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TREE_CASES = sorted(glob.glob(os.path.join(GOLDEN, "tree_*.npz")))
TREE_KEYS = ["index_map", "node_centers", "node_half_extents", "node_radii", "node_levels", "node_parents",
             "node_children", "node_ranges", "node_is_leaf"]


def _plan(pts, leaf, max_depth, theta, p=8):
    from electrodrive_gb300 import _lib

    return _lib.Plan(torch.as_tensor(pts).cuda(), leaf_size=leaf, max_depth=max_depth, mac_theta=theta,
                     expansion_order=p)


def _compare_tree(soa, want):
    for k in TREE_KEYS:
        got = soa[k].cpu().numpy()
        w = want[k] if isinstance(want, dict) else getattr(want, k)
        assert got.shape == w.shape, (k, got.shape, w.shape)
        assert np.array_equal(got.astype(w.dtype), w), f"{k} differs"


@pytest.mark.parametrize("path", TREE_CASES, ids=lambda p: os.path.basename(p)[5:-4])
def test_gpu_tree_and_lists_match_reference_fixture(cuda_lib, path):
    z = np.load(path)
    plan = _plan(z["points"], int(z["leaf_size"]), int(z["max_depth"]), float(z["theta"]))
    _compare_tree(plan.export_tree(), dict(z))
    p2p, m2l = plan.export_lists()
    assert np.array_equal(p2p.cpu().numpy(), z["p2p_pairs"])
    assert np.array_equal(m2l.cpu().numpy(), z["m2l_pairs"])
    assert plan.info.p2p_interactions == int(z["p2p_n_interactions"])


@pytest.mark.parametrize("kind,n,leaf,theta", [
    ("uniform", 200_000, 64, 0.5),
    ("clusters", 120_000, 32, 0.5),
    ("lattice", 60_000, 16, 0.6),
    ("sphere_f64", 80_000, 40, 0.5),
    ("coincident", 20_000, 8, 0.5),
])
def test_gpu_tree_and_lists_match_oracle_large(cuda_lib, oracle, kind, n, leaf, theta):
    rng = np.random.default_rng(hash(kind) % 2**31)
    if kind == "uniform":
        pts = rng.random((n, 3)).astype(np.float32)
    elif kind == "clusters":
        pts = np.concatenate([rng.normal(0.3, 0.01, (n // 2, 3)), rng.normal(0.7, 0.05, (n // 4, 3)),
                              rng.random((n - n // 2 - n // 4, 3))]).astype(np.float32)
    elif kind == "lattice":
        pts = (rng.integers(0, 40, (n, 3)) / 39.0).astype(np.float32)
    elif kind == "sphere_f64":
        v = rng.normal(size=(n, 3))
        pts = v / np.linalg.norm(v, axis=1, keepdims=True)
    else:
        pts = np.repeat(rng.random((n // 50, 3)), 50, axis=0).astype(np.float32)
    t = oracle.build_tree(pts, leaf, 32)
    lists = oracle.build_lists(t, theta)
    plan = _plan(pts, leaf, 32, theta)
    _compare_tree(plan.export_tree(), t)
    p2p, m2l = plan.export_lists()
    assert np.array_equal(p2p.cpu().numpy(), lists.p2p_pairs)
    assert np.array_equal(m2l.cpu().numpy(), lists.m2l_pairs)


def test_gpu_tree_empty_and_single(cuda_lib):
    plan = _plan(np.zeros((0, 3), np.float32), 64, 32, 0.5)
    assert plan.info.n_nodes == 0 and plan.info.n_p2p_pairs == 0
    plan1 = _plan(np.array([[0.25, 0.5, 0.75]], np.float32), 64, 32, 0.5)
    soa = plan1.export_tree()
    assert plan1.info.n_nodes == 1 and bool(soa["node_is_leaf"][0])
    p2p, m2l = plan1.export_lists()
    assert p2p.cpu().tolist() == [[0, 0]] and m2l.numel() == 0


def test_rebuild_lists_for_other_theta(cuda_lib, oracle):
    rng = np.random.default_rng(3)
    pts = rng.random((30_000, 3)).astype(np.float32)
    plan = _plan(pts, 32, 32, 0.5)
    t = oracle.build_tree(pts, 32, 32)
    for theta in (0.3, 0.7, 0.5):
        plan.rebuild_lists(theta)
        p2p, m2l = plan.export_lists()
        ol = oracle.build_lists(t, theta)
        assert np.array_equal(p2p.cpu().numpy(), ol.p2p_pairs)
        assert np.array_equal(m2l.cpu().numpy(), ol.m2l_pairs)


def test_public_tree_api(cuda_lib):
    from electrodrive_gb300.fmm3d import build_fmm_tree, build_interaction_lists

    z = np.load(os.path.join(GOLDEN, "tree_uniform4096_f32.npz"))
    tree = build_fmm_tree(torch.as_tensor(z["points"]), leaf_size=64)
    assert np.array_equal(tree.index_map.cpu().numpy(), z["index_map"])
    lists = build_interaction_lists(tree, mac_theta=0.5)
    assert lists.p2p_pairs == [tuple(x) for x in z["p2p_pairs"].tolist()]
    assert lists.num_m2l_pairs == z["m2l_pairs"].shape[0]
    q = torch.rand(4096, dtype=torch.float32)
    assert torch.equal(tree.map_to_original_order(tree.map_to_tree_order(q.cuda())).cpu(), q)
    assert tree.nodes[0].parent is None and tree.n_nodes == z["node_levels"].shape[0]
