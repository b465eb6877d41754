"""Restarted GMRES: the oracle pinned to the reference's own runs (CPU), and
the device solver against the same fixtures (GPU): same code, same number of
Arnoldi iterations, solution within 1e-8 relative (FP64)."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

Z = np.load(os.path.join(GOLDEN, "gmres_cases.npz"))
NAMES = sorted({k.split("__")[0] for k in Z.files})


def _case(name):
    if f"{name}__A" in Z.files:
        A = Z[f"{name}__A"]
    else:
        p, diag = Z[f"{name}__points"], Z[f"{name}__diag"]
        n = p.shape[0]
        d = np.sqrt(((p[:, None, :] - p[None, :, :]) ** 2).sum(-1))
        A = 1.0 / (n * (d + np.eye(n)))
        np.fill_diagonal(A, 0.0)
        A += np.diag(diag)
    restart, tol, maxiter, pc, iters, code, resid = Z[f"{name}__meta"]
    return A, Z[f"{name}__b"], Z[f"{name}__x"], int(restart), float(tol), int(maxiter), bool(pc), int(iters), int(code)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_gmres_matches_reference(name):
    from oracle import gmres_ref

    A, b, x_ref, restart, tol, maxiter, pc, iters, code = _case(name)
    pinv = 1.0 / np.diag(A) if pc else None
    x, info = gmres_ref.gmres_restart(lambda v: A @ v, b, pinv, restart, tol, maxiter)
    assert info["code"] == code and info["iters"] == iters
    assert np.linalg.norm(x - x_ref) <= 1e-10 * np.linalg.norm(x_ref)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("graph", [False, True])
def test_device_gmres_matches_reference(cuda_lib, name, graph):
    from electrodrive_gb300.core.bem_solver import gmres_restart, setup_preconditioner

    A, b, x_ref, restart, tol, maxiter, pc, iters, code = _case(name)
    At = torch.as_tensor(A, device="cuda")
    out = torch.empty(A.shape[0], dtype=torch.float64, device="cuda")

    class Op:
        capturable = True

        def __call__(self, v):
            torch.mv(At, v, out=out)
            return out

    M = setup_preconditioner("jacobi", A_diag=torch.diag(At)) if pc else None
    x, info = gmres_restart(Op() if graph else (lambda v: At @ v), torch.as_tensor(b, device="cuda"), M=M,
                            restart=restart, tol=tol, maxiter=maxiter, use_graph=graph)
    assert info["code"] == code and info["iters"] == iters
    x = x.cpu().numpy()
    if code == 0:
        assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
        assert np.linalg.norm(A @ x - b) <= info["tol_abs"] * (1 + 1e-9)
    else:
        assert np.linalg.norm(x - x_ref) <= 1e-6 * np.linalg.norm(x_ref)


@pytest.mark.gpu
def test_device_gmres_fp32_and_host_vectors(cuda_lib):
    from electrodrive_gb300.core.bem_solver import gmres_restart

    A, b, x_ref, *_ = _case("nonsym120_jacobi")
    Af = torch.as_tensor(A, dtype=torch.float32)
    x, info = gmres_restart(lambda v: Af @ v, torch.as_tensor(b, dtype=torch.float32), restart=20, tol=1e-5,
                            maxiter=200, precond="jacobi", A_diag=torch.diag(Af))
    assert x.device.type == "cpu" and x.dtype == torch.float32
    assert info["success"] and info["used_preconditioner"]
    assert np.linalg.norm(x.double().numpy() - x_ref) <= 1e-4 * np.linalg.norm(x_ref)


@pytest.mark.gpu
def test_device_gmres_failure_codes(cuda_lib):
    from electrodrive_gb300.core.bem_solver import gmres_restart

    n = 100
    b = torch.ones(n, dtype=torch.float64, device="cuda")
    x, info = gmres_restart(lambda v: v * float("nan"), b, restart=5, maxiter=10)
    assert not info["success"] and info["code"] == 3
    x, info = gmres_restart(lambda v: 2 * v, b, restart=5, maxiter=10, live_control_poll_fn=lambda: {"terminate": True})
    assert info["code"] in (0, 2)
    with pytest.raises(ValueError):
        gmres_restart(lambda v: v, b, restart=0)


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [False, True])
def test_device_gmres_early_exit(cuda_lib, graph):
    """early_exit (not in the reference): cycles end on the inner estimate, the
    true residual still decides, and the answer is the converged one."""
    from electrodrive_gb300.core.bem_solver import gmres_restart, setup_preconditioner

    A, b, x_ref, restart, tol, maxiter, pc, iters, code = _case("bemlike300_jacobi")
    At = torch.as_tensor(A, device="cuda")
    out = torch.empty(A.shape[0], dtype=torch.float64, device="cuda")

    class Op:
        capturable = True

        def __call__(self, v):
            torch.mv(At, v, out=out)
            return out

    M = setup_preconditioner("jacobi", A_diag=torch.diag(At))
    x, info = gmres_restart(Op(), torch.as_tensor(b, device="cuda"), M=M, restart=restart, tol=tol,
                            maxiter=maxiter, use_graph=graph, early_exit=4)
    assert info["code"] == 0 and info["iters"] < iters
    x = x.cpu().numpy()
    assert np.linalg.norm(A @ x - b) <= info["tol_abs"] * (1 + 1e-9)
    assert np.linalg.norm(x - x_ref) <= 1e-6 * np.linalg.norm(x_ref)


@pytest.mark.gpu
def test_device_gmres_graph_from_the_second_request(cuda_lib):
    """A step sequence runs as direct launches the first time it is asked for
    and from a captured graph afterwards (here: a second solve with the same
    operator); the iterates are identical either way."""
    from electrodrive_gb300.core import bem_solver as bs

    A, b, x_ref, restart, tol, maxiter, pc, iters, code = _case("bemlike300_jacobi")
    At = torch.as_tensor(A, device="cuda")
    out = torch.empty(A.shape[0], dtype=torch.float64, device="cuda")

    class Op:
        capturable = True

        def __call__(self, v):
            torch.mv(At, v, out=out)
            return out

    op, bt = Op(), torch.as_tensor(b, device="cuda")
    runs = []
    for _ in range(2):
        x, info = bs.gmres_restart(op, bt, restart=restart, tol=tol, maxiter=maxiter, precond="jacobi",
                                   A_diag=torch.diag(At), use_graph=True, early_exit=4)
        runs.append((x.clone(), info))
    (x1, i1), (x2, i2) = runs
    assert i1["code"] == 0 and i1["iters"] == i2["iters"]
    assert torch.equal(x1, x2)
    assert any(ws["graphs"] for ws in bs._GRAPH_CACHE[op].values())


def test_jacobi_fallback_converges_or_reports_failure():
    """core.bem.jacobi_fallback_solve, the reference's damped-Jacobi last
    resort (electrodrive/core/bem.py:1156-1251), on CPU tensors: a diagonally
    dominant system converges to tol * max(|b|, 1); a system whose Jacobi
    iteration diverges ends with a non-finite residual and success False."""
    import torch

    from electrodrive_gb300.core.bem import jacobi_fallback_solve

    g = torch.Generator().manual_seed(0)
    n = 60
    M = torch.rand(n, n, generator=g, dtype=torch.float64) * 0.01
    M += torch.diag(torch.full((n,), 2.0, dtype=torch.float64))
    b = torch.rand(n, generator=g, dtype=torch.float64)
    x, info = jacobi_fallback_solve(lambda v: M @ v, b, torch.diagonal(M).clone(), maxiter=256, tol=1e-10,
                                    omega=0.8)
    assert info["success"] and info["solver"] == "jacobi_fallback"
    assert float(torch.linalg.norm(b - M @ x)) <= 1e-10 * max(float(torch.linalg.norm(b)), 1.0)
    D = torch.ones(n, n, dtype=torch.float64) + torch.eye(n, dtype=torch.float64)
    x, info = jacobi_fallback_solve(lambda v: D @ v, b, torch.diagonal(D).clone(), maxiter=2000, tol=1e-10,
                                    omega=0.8)
    assert not info["success"] and not np.isfinite(info["resid"])
