"""Triangle quadrature rules (electrodrive/core/bem_quadrature.py:79-344).

Host-side NumPy versions of the reference's rule constructors, kept for API
compatibility (they build rules, they do not integrate anything).  The
solver evaluates the same rules on the GPU (``bem_near``).
"""
from __future__ import annotations

import math
from typing import Optional, Tuple

import numpy as np

from ..utils.config import K_E


def _tri(vertices) -> np.ndarray:
    v = np.asarray(vertices, dtype=float)
    if v.shape != (3, 3):
        raise ValueError(f"vertices must have shape (3, 3), got {v.shape}")
    return v


def _triangle_area(v: np.ndarray) -> float:
    return 0.5 * float(np.linalg.norm(np.cross(v[1] - v[0], v[2] - v[0])))


def standard_triangle_quadrature(vertices, order: int = 2) -> Tuple[np.ndarray, np.ndarray]:
    verts = _tri(vertices)
    if order <= 1:
        bary = np.array([[1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0]])
        w_ref = np.array([1.0])
    elif order == 2:
        a, b = 2.0 / 3.0, 1.0 / 6.0
        bary = np.array([[a, b, b], [b, a, b], [b, b, a]])
        w_ref = np.full(3, 1.0 / 3.0)
    else:
        raise NotImplementedError(f"Triangle quadrature of order {order} is not implemented; supported orders are 1 and 2.")
    area = _triangle_area(verts)
    if area <= 0.0:
        return np.mean(verts, axis=0, keepdims=True), np.zeros_like(w_ref)
    pts = bary[:, 0:1] * verts[0:1, :] + bary[:, 1:2] * verts[1:2, :] + bary[:, 2:3] * verts[2:3, :]
    return pts, w_ref * area


def reference_triangle_quadrature(order: int = 2) -> Tuple[np.ndarray, np.ndarray]:
    if order <= 1:
        return np.array([[1.0 / 3.0, 1.0 / 3.0]]), np.array([0.5])
    if order == 2:
        return np.array([[2.0 / 3.0, 1.0 / 6.0], [1.0 / 6.0, 2.0 / 3.0], [1.0 / 6.0, 1.0 / 6.0]]), np.full(3, 1.0 / 6.0)
    raise NotImplementedError(f"Reference triangle quadrature of order {order} is not implemented; "
                              "supported orders are 1 and 2.")


def near_singular_quadrature(target, panel_vertices, method: str = "telles", order: int = 2, *,
                             max_depth: Optional[int] = None) -> Tuple[np.ndarray, np.ndarray]:
    verts = _tri(panel_vertices)
    tgt = np.asarray(target, dtype=float).reshape(3)
    depth = max_depth if max_depth is not None else (4 if method.lower() == "telles" else 1)
    if depth <= 0:
        return standard_triangle_quadrature(verts, order=order)
    tris = [verts]
    for _ in range(depth):
        cents = np.array([t.mean(axis=0) for t in tris])
        idx = int(np.argmin(np.linalg.norm(cents - tgt[None, :], axis=1)))
        v0, v1, v2 = tris.pop(idx)
        m01, m12, m20 = 0.5 * (v0 + v1), 0.5 * (v1 + v2), 0.5 * (v2 + v0)
        tris += [np.stack([v0, m01, m20]), np.stack([m01, v1, m12]), np.stack([m20, m12, v2]), np.stack([m01, m12, m20])]
    pts, ws = zip(*(standard_triangle_quadrature(t, order=order) for t in tris))
    return np.vstack(pts), np.concatenate(ws)


def self_integral_correction(area) -> float:
    a = float(area)
    return 0.0 if a <= 0.0 else 2.0 * math.pi * K_E * math.sqrt(a / math.pi)


__all__ = ["standard_triangle_quadrature", "reference_triangle_quadrature", "near_singular_quadrature",
           "self_integral_correction"]
