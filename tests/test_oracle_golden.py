"""Pin the CPU oracle against fixtures written by the reference itself.

The fixtures in tests/golden/ come from tests/golden/make_golden.py, which
runs the reference's build_fmm_tree / build_interaction_lists /
apply_p2p_cpu_tiled / LaplaceFmm3D / bem_matvec_gpu.  The oracle's tree and
interaction lists must match bit for bit; potentials within the tolerances
the reference's own tests use (kernels_cpu P2P: 1e-6 in FP32).
"""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

TREE_CASES = sorted(glob.glob(os.path.join(GOLDEN, "tree_*.npz")))
FMM_CASES = sorted(glob.glob(os.path.join(GOLDEN, "fmm_*.npz")))
TREE_KEYS = ["index_map", "node_centers", "node_half_extents", "node_radii", "node_levels", "node_parents",
             "node_children", "node_ranges", "node_is_leaf"]


@pytest.mark.parametrize("path", TREE_CASES, ids=lambda p: os.path.basename(p)[5:-4])
def test_oracle_tree_and_lists_bit_exact(oracle, path):
    z = np.load(path)
    t = oracle.build_tree(z["points"], int(z["leaf_size"]), int(z["max_depth"]))
    for k in TREE_KEYS:
        got = getattr(t, k)
        want = z[k]
        assert got.shape == want.shape, k
        assert np.array_equal(got.astype(want.dtype), want), f"{k} differs"
    # the oracle keeps float data in the tree dtype
    assert t.node_centers.dtype == z["points"].dtype
    lists = oracle.build_lists(t, float(z["theta"]))
    assert np.array_equal(lists.p2p_pairs, z["p2p_pairs"])
    assert np.array_equal(lists.m2l_pairs, z["m2l_pairs"])


@pytest.mark.parametrize("path", TREE_CASES, ids=lambda p: os.path.basename(p)[5:-4])
def test_oracle_p2p_matches_reference(oracle, path):
    z = np.load(path)
    t = oracle.build_tree(z["points"], int(z["leaf_size"]), int(z["max_depth"]))
    lists = oracle.build_lists(t, float(z["theta"]))
    eps = float(np.finfo(z["points"].dtype).eps)
    phi = oracle.p2p(t.points_tree, z["charges"][t.index_map], t.node_ranges, lists.p2p_pairs, eps)
    ref = z["p2p_potential_tree"].astype(np.float64)
    tol = 1e-12 if z["points"].dtype == np.float64 else 1e-6
    assert np.linalg.norm(phi - ref) <= tol * np.linalg.norm(ref)


def test_oracle_detects_a_planted_tree_error(oracle):
    """A checker that cannot fail checks nothing: perturb one point by one ulp."""
    z = np.load(os.path.join(GOLDEN, "tree_lattice2000_f32.npz"))
    pts = z["points"].copy()
    t0 = oracle.build_tree(pts, int(z["leaf_size"]), int(z["max_depth"]))
    # find a point lying exactly on a splitting plane of an internal node
    hit = None
    for i in np.nonzero(~t0.node_is_leaf)[0]:
        s, e = t0.node_ranges[i]
        idx = t0.index_map[s:e]
        on = np.nonzero(pts[idx, 0] == t0.node_centers[i, 0])[0]
        if on.size:
            hit = idx[on[0]]
            break
    assert hit is not None
    # strict '>' sends it to the lower child; one ulp up must change the tree
    pts[hit, 0] = np.nextafter(pts[hit, 0], np.float32(2.0))
    t1 = oracle.build_tree(pts, int(z["leaf_size"]), int(z["max_depth"]))
    assert not np.array_equal(t1.index_map, z["index_map"])


@pytest.mark.parametrize("path", FMM_CASES, ids=lambda p: os.path.basename(p)[4:-4])
def test_oracle_fmm_against_reference_fixtures(oracle, path):
    """Oracle FP64 FMM vs the reference's dense operator and the reference FMM.

    The reference FMM's own error vs its dense operator (recorded in the
    fixture) is the budget: the oracle must be at least as close to the dense
    operator, and within that budget (+1e-5) of the reference FMM.
    """
    z = np.load(path)
    pts, sigma, areas, si = z["points"], z["sigma"], z["areas"], z["self_integrals"]
    t = oracle.build_tree(pts, int(z["leaf_size"]), 32)
    lists = oracle.build_lists(t, float(z["theta"]))
    v = oracle.fmm_matvec(t, lists, pts, sigma, areas, si, p=int(z["p"]))
    dense = z["v_dense_reference"].astype(np.float64)
    ref_fmm = z["v_fmm_reference"].astype(np.float64)
    nd = np.linalg.norm(dense)
    ref_err = np.linalg.norm(ref_fmm - dense) / nd
    our_err = np.linalg.norm(v - dense) / nd
    assert our_err < 1e-5, our_err
    assert our_err <= ref_err
    assert np.linalg.norm(v - ref_fmm) / nd <= ref_err + 1e-5
    # the oracle's dense restatement reproduces the reference dense operator
    vd = oracle.dense_matvec(pts, sigma, areas, si)
    assert np.linalg.norm(vd - dense) / nd < 1e-6


def test_oracle_fmm_vs_direct_sum(oracle):
    rng = np.random.default_rng(5)
    n = 5000
    pts = rng.random((n, 3)).astype(np.float32)
    q = rng.uniform(-1, 1, n)
    t = oracle.build_tree(pts, 64, 32)
    lists = oracle.build_lists(t, 0.5)
    v = oracle.fmm_matvec(t, lists, pts, q, np.ones(n), None, p=8, ke=1.0)
    d = oracle.direct(pts, q)
    assert np.linalg.norm(v - d) / np.linalg.norm(d) < 1e-6
    # the reference's swapped M2L unpacking changes only non-symmetric pairs
    v2 = oracle.fmm_matvec(t, lists, pts, q, np.ones(n), None, p=8, ke=1.0, reference_pair_order=True)
    assert np.linalg.norm(v2 - d) / np.linalg.norm(d) < 1e-5


def test_oracle_empty_and_single(oracle):
    t = oracle.build_tree(np.zeros((0, 3), np.float32), 64, 32)
    assert t.n_nodes == 0
    lists = oracle.build_lists(t, 0.5)
    assert lists.p2p_pairs.shape == (0, 2) and lists.m2l_pairs.shape == (0, 2)
    t1 = oracle.build_tree(np.array([[0.1, 0.2, 0.3]], np.float32), 64, 32)
    assert t1.n_nodes == 1 and bool(t1.node_is_leaf[0])
    l1 = oracle.build_lists(t1, 0.5)
    assert l1.p2p_pairs.tolist() == [[0, 0]]
