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
