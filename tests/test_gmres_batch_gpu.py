"""Batched GMRES (edfmm_bgmres_*, core.bem_solver.gmres_batched).

Each instance of a block-diagonal system must follow the single-instance
solver: with the single solver's estimate checked after every step
(early_exit=1) both stop at the same steps, so the per-instance iteration
counts are equal and the solutions agree to rounding (the reductions are
partitioned differently).  An instance given a negative tolerance is left
untouched, and FP32 runs reach the requested residual per instance.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SIZES = [37, 300, 1, 129, 64, 500]


def _blocks(dtype, seed=0):
    rng = np.random.default_rng(seed)
    mats = []
    for n in SIZES:
        a = np.eye(n) * rng.uniform(2.0, 4.0, n) + rng.normal(size=(n, n)) / np.sqrt(n)
        mats.append(torch.as_tensor(a, dtype=dtype, device="cuda"))
    segs = np.concatenate([[0], np.cumsum(SIZES)]).tolist()
    b = torch.as_tensor(rng.normal(size=segs[-1]), dtype=dtype, device="cuda")

    def A(x):
        return torch.cat([mats[k] @ x[segs[k]:segs[k + 1]] for k in range(len(SIZES))])

    diag = torch.cat([torch.diagonal(m) for m in mats])
    return mats, segs, b, A, diag


@pytest.mark.parametrize("restart", [10, 64])
def test_batched_matches_single_instance_fp64(cuda_lib, restart):
    from electrodrive_gb300.core.bem_solver import gmres_batched, gmres_restart

    mats, segs, b, A, diag = _blocks(torch.float64)
    tol = 1e-10
    x, info = gmres_batched(A, b, segs, restart=restart, tol=tol, maxiter=400, A_diag=diag, check_every=4)
    assert info["code"] == 0 and all(info["converged"]), info
    for k, m in enumerate(mats):
        s, e = segs[k], segs[k + 1]
        if e - s == 1:
            # the one-row system ends in a lucky breakdown at its first step,
            # which the batched solver keeps (the single-instance solver, as the
            # reference, drops that column and reports stagnation)
            assert info["instance_iters"][k] == 1
            assert abs(float(x[s] - b[s] / m[0, 0])) <= 1e-14 * abs(float(b[s] / m[0, 0]))
            continue
        xs, si = gmres_restart(lambda v: m @ v, b[s:e], restart=restart, tol=tol, maxiter=400, precond="jacobi",
                               A_diag=diag[s:e], use_graph=False, early_exit=1)
        assert si["code"] == 0
        assert info["instance_iters"][k] == si["iters"], k
        assert float(torch.linalg.norm(x[s:e] - xs) / torch.linalg.norm(xs)) < 1e-9, k
        r = float(torch.linalg.norm(b[s:e] - m @ x[s:e]) / torch.linalg.norm(b[s:e]))
        assert r <= tol * 1.01, k
    assert info["iters"] >= max(info["instance_iters"])  # the shared steps cover the slowest instance


def test_negative_tolerance_leaves_instance_untouched(cuda_lib):
    from electrodrive_gb300.core.bem_solver import gmres_batched

    mats, segs, b, A, diag = _blocks(torch.float64, seed=1)
    x0 = torch.full_like(b, 0.25)
    tol = torch.full((len(SIZES),), 1e-8, dtype=torch.float64)
    tol[1] = -1.0
    x, info = gmres_batched(A, b, segs, restart=40, tol=tol, maxiter=300, A_diag=diag, x0=x0)
    assert info["code"] == 0
    assert info["instance_iters"][1] == 0
    assert torch.equal(x[segs[1]:segs[2]], x0[segs[1]:segs[2]])
    for k in (0, 2, 3, 4, 5):
        s, e = segs[k], segs[k + 1]
        r = float(torch.linalg.norm(b[s:e] - mats[k] @ x[s:e]) / torch.linalg.norm(b[s:e] - mats[k] @ x0[s:e]))
        assert r <= 1e-8 * 1.01, k


def test_batched_fp32_reaches_tolerance_with_graphs(cuda_lib):
    from electrodrive_gb300.core.bem_solver import gmres_batched

    mats, segs, b, A, diag = _blocks(torch.float32, seed=2)
    x, info = gmres_batched(A, b, segs, restart=30, tol=1e-5, maxiter=300, A_diag=diag, use_graph=True)
    assert info["code"] == 0
    for k, m in enumerate(mats):
        s, e = segs[k], segs[k + 1]
        r = float(torch.linalg.norm((b[s:e] - m @ x[s:e]).double()) / torch.linalg.norm(b[s:e].double()))
        assert r <= 2e-5, k
