"""NumPy restatement of the reference's restarted GMRES (test infrastructure).

Follows electrodrive/core/bem_solver.py:125-920: left preconditioner,
modified Gram-Schmidt Arnoldi (:536-541), Givens rotations with the
denominator < 1e-14 rule (:590-616), full restart cycles (the inner estimate
never ends a cycle, :650-655), triangular solve (:762-769), true-residual
convergence test at the end of each cycle (:776-865), tol_abs rule (:407),
codes 0/1/2/3/5/6/7 and the one-time retry without preconditioner for
N <= 512 (:472).  Only used by tests/ as the checker of the GPU solver.
"""
from __future__ import annotations

import math

import numpy as np


def gmres_restart(A, b, pinv=None, restart=80, tol=1e-8, maxiter=500, x0=None, _retried=False):
    b = np.asarray(b, dtype=np.float64)
    N = b.shape[0]
    M = (lambda v: v) if pinv is None else (lambda v: pinv * v)
    used = pinv is not None
    can_retry = used and not _retried and N <= 512

    def retry():
        return gmres_restart(A, b, None, restart, tol, maxiter, x0, _retried=True)

    x = np.zeros(N) if x0 is None else np.array(x0, dtype=np.float64)
    r_true = b - A(x)
    r_true_norm = float(np.linalg.norm(r_true))
    if not math.isfinite(r_true_norm):
        return x, dict(iters=0, success=False, code=3, resid=r_true_norm)
    r = M(r_true)
    beta = float(np.linalg.norm(r))
    if not math.isfinite(beta):
        if used and not _retried:
            return retry()
        return x, dict(iters=0, success=False, code=7, resid=r_true_norm)
    r_norm = beta
    init_true = r_true_norm if r_true_norm > 1e-16 else 1.0
    tol_abs = max(tol * init_true, tol * 1e-12, 1e-12)
    total = 0
    max_cycles = max(1, (maxiter + restart - 1) // restart)
    for _cycle in range(max_cycles):
        V = [r / beta]
        H = np.zeros((restart + 1, restart))
        g = np.zeros(restart + 1)
        g[0] = beta
        rot = []
        j = 0
        while j < restart and total < maxiter:
            w = M(A(V[j]))
            total += 1
            for i in range(j + 1):
                H[i, j] = float(np.dot(V[i], w))
                w = w - H[i, j] * V[i]
            H[j + 1, j] = float(np.linalg.norm(w))
            hn = H[j + 1, j]
            if not math.isfinite(hn) or hn <= 0.0:
                if can_retry:
                    return retry()
                break
            V.append(w / hn)
            for ig, (c, s) in enumerate(rot):
                t = c * H[ig, j] + s * H[ig + 1, j]
                H[ig + 1, j] = -s * H[ig, j] + c * H[ig + 1, j]
                H[ig, j] = t
            den = math.sqrt(H[j, j] ** 2 + H[j + 1, j] ** 2)
            if den < 1e-14 or not math.isfinite(den):
                c, s = 1.0, 0.0
            else:
                c, s = H[j, j] / den, H[j + 1, j] / den
            rot.append((c, s))
            H[j, j] = c * H[j, j] + s * H[j + 1, j]
            H[j + 1, j] = 0.0
            g[j], g[j + 1] = c * g[j], -s * g[j]
            r_norm = abs(g[j + 1])
            if not math.isfinite(r_norm):
                if can_retry:
                    return retry()
                return x, dict(iters=total, success=False, code=5, resid=r_norm)
            j += 1
        m = j
        if m == 0:
            if can_retry:
                return retry()
            return x, dict(iters=total, success=False, code=2, resid=r_norm)
        y = np.zeros(m)
        for i in range(m - 1, -1, -1):
            y[i] = (g[i] - H[i, i + 1:m] @ y[i + 1:m]) / H[i, i]
        x = x + np.stack(V[:m], axis=1) @ y
        r_true = b - A(x)
        r_true_norm = float(np.linalg.norm(r_true))
        if not math.isfinite(r_true_norm):
            if can_retry:
                return retry()
            return x, dict(iters=total, success=False, code=6, resid=r_true_norm)
        r = M(r_true)
        beta = float(np.linalg.norm(r))
        r_norm = beta
        if r_true_norm <= tol_abs:
            return x, dict(iters=total, success=True, code=0, resid=r_true_norm, tol_abs=tol_abs)
        if total >= maxiter:
            break
    if can_retry:
        return retry()
    return x, dict(iters=total, success=False, code=1, resid=r_norm, tol_abs=tol_abs)
