"""FMM evaluation at arbitrary targets (bem_potential_targets by FMM).

Lists between a source tree and a separate target tree are bit-identical to
the reference's build_interaction_lists(source_tree, target_tree) on the
fixtures written by it (tests/golden/make_golden.py, group "targets"); the
potential agrees with the FP64 direct sum to the FMM's accuracy at p = 8
(1e-5 relative) and with the dense evaluation.
"""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
Z = np.load(os.path.join(GOLDEN, "targets_cases.npz"))
CASES = sorted({k.split("__")[0] for k in Z.files})


@pytest.mark.parametrize("name", CASES)
def test_two_tree_lists_match_reference(cuda_lib, name):
    from electrodrive_gb300._lib import Plan

    leaf, theta = Z[f"{name}__meta"]
    if int(Z[f"{name}__target_leaf"][0]) != int(leaf):
        pytest.skip("plan.targets builds the target tree at the source leaf size")
    src = torch.as_tensor(Z[f"{name}__sources"], device="cuda")
    tgt = torch.as_tensor(Z[f"{name}__targets"], device="cuda")
    plan = Plan(src, leaf_size=int(leaf), mac_theta=float(theta))
    tg = plan.targets(tgt)
    p2p, m2l = tg.export_lists()
    assert np.array_equal(p2p.cpu().numpy(), Z[f"{name}__p2p_pairs"])
    assert np.array_equal(m2l.cpu().numpy(), Z[f"{name}__m2l_pairs"])


def _direct(tgt, src, q):
    out = np.empty(tgt.shape[0])
    for i in range(0, tgt.shape[0], 200):
        d = np.sqrt(((tgt[i:i + 200, None, :] - src[None, :, :]) ** 2).sum(-1))
        out[i:i + 200] = (q[None, :] / d).sum(1)
    return out


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_target_potential_matches_direct_sum(cuda_lib, dtype):
    from electrodrive_gb300._lib import Plan

    rng = np.random.default_rng(5)
    src = rng.random((20000, 3))
    tgt = rng.random((3000, 3)) * 1.6 - 0.3  # inside, around and outside the sources
    sigma = rng.uniform(-1, 1, src.shape[0])
    areas = rng.uniform(0.5, 1.5, src.shape[0]) / src.shape[0]
    T = lambda x: torch.as_tensor(x, dtype=dtype, device="cuda")
    plan = Plan(T(src), leaf_size=64, expansion_order=8)
    tg = plan.targets(T(tgt))
    v = tg.potential(T(sigma), T(areas), k_e=1.0).double().cpu().numpy()
    npdt = np.float32 if dtype == torch.float32 else np.float64
    q = (sigma.astype(npdt).astype(np.float64) * areas.astype(npdt).astype(np.float64))
    ref = _direct(tgt.astype(npdt).astype(np.float64), src.astype(npdt).astype(np.float64), q)
    assert np.linalg.norm(v - ref) <= 1e-5 * np.linalg.norm(ref)
    near_only = tg.potential(T(sigma), T(areas), k_e=1.0, flags=2).double().cpu().numpy()
    far_only = tg.potential(T(sigma), T(areas), k_e=1.0, flags=4).double().cpu().numpy()
    assert np.linalg.norm(near_only + far_only - v) <= 1e-6 * np.linalg.norm(ref)


def test_bem_potential_targets_fmm_matches_dense(cuda_lib):
    from electrodrive_gb300.core.bem_kernel import bem_potential_targets

    rng = np.random.default_rng(6)
    c = torch.as_tensor(rng.normal(size=(15000, 3)), device="cuda")
    a = torch.as_tensor(rng.uniform(0.5, 1.5, 15000) / 15000, device="cuda")
    s = torch.as_tensor(rng.uniform(-1, 1, 15000), device="cuda")
    x = torch.as_tensor(rng.normal(size=(2000, 3)) * 2.0, device="cuda")
    vd = bem_potential_targets(x, c, a, s, method="dense")
    vf = bem_potential_targets(x, c, a, s, method="fmm")
    assert float(torch.linalg.norm(vf - vd) / torch.linalg.norm(vd)) < 1e-5


@pytest.mark.parametrize("name", CASES)
def test_public_two_tree_lists_match_reference(cuda_lib, name):
    """build_interaction_lists(source_tree, target_tree) through the public
    Python API, each tree built with its own leaf size."""
    from electrodrive_gb300.fmm3d import build_fmm_tree, build_interaction_lists
    from electrodrive_gb300.fmm3d.interaction_lists import verify_interaction_lists

    leaf, theta = Z[f"{name}__meta"]
    tleaf = int(Z[f"{name}__target_leaf"][0])
    stree = build_fmm_tree(torch.as_tensor(Z[f"{name}__sources"], device="cuda"), leaf_size=int(leaf))
    ttree = build_fmm_tree(torch.as_tensor(Z[f"{name}__targets"], device="cuda"), leaf_size=tleaf)
    assert np.array_equal(ttree.index_map.cpu().numpy(), Z[f"{name}__target_index_map"])
    lists = build_interaction_lists(stree, ttree, mac_theta=float(theta))
    assert not lists.same_tree
    assert np.array_equal(np.asarray(lists.p2p_pairs, dtype=np.int32).reshape(-1, 2), Z[f"{name}__p2p_pairs"])
    assert np.array_equal(np.asarray(lists.m2l_pairs, dtype=np.int32).reshape(-1, 2), Z[f"{name}__m2l_pairs"])
    verify_interaction_lists(stree, ttree, lists)


@pytest.mark.parametrize("name", CASES)
def test_public_two_tree_stages_match_direct_sums(cuda_lib, name):
    """apply_p2p_gpu and p2m -> m2m -> m2l -> l2l -> l2p between two trees:
    the near part equals the sum over the listed leaf pairs (no self
    exclusion between distinct trees) and near + far equals the direct sum to
    the FMM's accuracy at p = 8."""
    from electrodrive_gb300.fmm3d import FmmConfig, build_fmm_tree, build_interaction_lists
    from electrodrive_gb300.fmm3d.kernels_gpu import apply_p2p_gpu
    from electrodrive_gb300.fmm3d.multipole_operators import l2l, l2p, m2l, m2m, p2m

    leaf, theta = Z[f"{name}__meta"]
    tleaf = int(Z[f"{name}__target_leaf"][0])
    src = Z[f"{name}__sources"]
    tgt = Z[f"{name}__targets"]
    dt = torch.float32 if src.dtype == np.float32 else torch.float64
    stree = build_fmm_tree(torch.as_tensor(src, device="cuda"), leaf_size=int(leaf))
    ttree = build_fmm_tree(torch.as_tensor(tgt, device="cuda"), leaf_size=tleaf)
    lists = build_interaction_lists(stree, ttree, mac_theta=float(theta))
    q = np.random.default_rng(7).uniform(-1, 1, src.shape[0]).astype(src.dtype)
    q_dev = torch.as_tensor(q, device="cuda")
    # near field over the listed leaf pairs, tree orders of both trees
    res = apply_p2p_gpu(stree, ttree, stree.map_to_tree_order(q_dev), lists)
    assert res.n_pairs == lists.num_p2p_pairs
    sp = src.astype(np.float64)[stree.index_map.cpu().numpy()]
    tp = tgt.astype(np.float64)[ttree.index_map.cpu().numpy()]
    qt = q.astype(np.float64)[stree.index_map.cpu().numpy()]
    sr = stree.node_ranges.cpu().numpy()
    tr = ttree.node_ranges.cpu().numpy()
    eps = float(np.finfo(src.dtype).eps)
    ref = np.zeros(tgt.shape[0])
    for s_node, t_node in np.asarray(lists.p2p_pairs):
        xs, qs = sp[sr[s_node, 0]:sr[s_node, 1]], qt[sr[s_node, 0]:sr[s_node, 1]]
        xt = tp[tr[t_node, 0]:tr[t_node, 1]]
        d = np.sqrt(((xt[:, None, :] - xs[None, :, :]) ** 2).sum(-1))
        ref[tr[t_node, 0]:tr[t_node, 1]] += (qs[None, :] / np.maximum(d, eps)).sum(1)
    near = res.potential.double().cpu().numpy()
    tol = 2e-6 if dt == torch.float32 else 1e-12
    assert np.linalg.norm(near - ref) <= tol * np.linalg.norm(ref)
    # far field through the tree-level stages, then near + far vs the direct sum
    cfg = FmmConfig(expansion_order=8, mac_theta=float(theta), leaf_size=int(leaf))
    M = m2m(stree, p2m(stree, q_dev, cfg), cfg)
    L = m2l(stree, ttree, M, cfg, lists=lists)
    assert L.tree is ttree and L.data.shape[0] == ttree.n_nodes
    far = l2p(ttree, l2l(ttree, L, cfg), cfg).double().cpu().numpy()
    d = np.sqrt(((tp[:, None, :] - src.astype(np.float64)[None, :, :]) ** 2).sum(-1))
    direct = (q.astype(np.float64)[None, :] / d).sum(1)
    assert np.linalg.norm(near + far - direct) <= 1e-5 * np.linalg.norm(direct)
