"""Panel meshes (electrodrive/core/bem_mesh.py:13-212) plus an icosphere.

``generate_mesh(spec, target_h)`` reproduces the reference's tensor-grid
plane patch, UV sphere and torus (same resolution heuristics, vertex and
triangle order, degenerate-panel drop, normals), vectorised with NumPy.
``icosphere(subdivisions, radius, center)`` builds the geodesic sphere the
reference does not have (20 * 4^s flat triangles; s = 4 gives 5,120 panels):
icosahedron vertices on the unit sphere, each subdivision splits every face
into four through edge midpoints pushed back onto the sphere.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass
from typing import Any, Dict, List, Optional, Tuple

import numpy as np


@dataclass
class TriMesh:
    vertices: np.ndarray
    triangles: np.ndarray
    centroids: np.ndarray
    normals: np.ndarray
    areas: np.ndarray
    conductor_ids: np.ndarray

    @property
    def n_panels(self) -> int:
        return int(self.triangles.shape[0])

    @property
    def panel_vertices(self) -> np.ndarray:
        return self.vertices[self.triangles]


def _finish(vertices: np.ndarray, triangles: np.ndarray, cids: np.ndarray) -> TriMesh:
    v0, v1, v2 = vertices[triangles[:, 0]], vertices[triangles[:, 1]], vertices[triangles[:, 2]]
    centroids = (v0 + v1 + v2) / 3.0
    cross = np.cross(v1 - v0, v2 - v0)
    areas = 0.5 * np.linalg.norm(cross, axis=1)
    mask = areas > 1e-16
    if (~mask).any():
        triangles, centroids, cross, areas, cids = triangles[mask], centroids[mask], cross[mask], areas[mask], cids[mask]
    normals = cross / (2.0 * areas[:, None] + 1e-30)
    return TriMesh(vertices, triangles, centroids, normals, areas, cids)


def _mesh_plane_patch(z: float, L: float, n: int) -> Tuple[np.ndarray, np.ndarray]:
    x = np.linspace(-L / 2.0, L / 2.0, n + 1)
    y = np.linspace(-L / 2.0, L / 2.0, n + 1)
    xx, yy = np.meshgrid(x, y, indexing="ij")
    vertices = np.stack([xx.ravel(), yy.ravel(), np.full(xx.size, z)], axis=1)
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    idx = (i * (n + 1) + j).ravel()
    t1 = np.stack([idx, idx + 1, idx + (n + 1)], axis=1)
    t2 = np.stack([idx + 1, idx + (n + 2), idx + (n + 1)], axis=1)
    tris = np.stack([t1, t2], axis=1).reshape(-1, 3)
    return vertices, tris.astype(np.int32)


def _mesh_sphere(center: np.ndarray, radius: float, n_theta: int, n_phi: int) -> Tuple[np.ndarray, np.ndarray]:
    theta = np.linspace(0.0, np.pi, n_theta)
    phi = np.linspace(0.0, 2.0 * np.pi, n_phi, endpoint=False)
    t, p = np.meshgrid(theta, phi, indexing="ij")
    vertices = np.stack([center[0] + radius * np.sin(t) * np.cos(p), center[1] + radius * np.sin(t) * np.sin(p),
                         center[2] + radius * np.cos(t)], axis=-1).reshape(-1, 3)
    i, j = np.meshgrid(np.arange(n_theta - 1), np.arange(n_phi), indexing="ij")
    jn = (j + 1) % n_phi
    a, b = i * n_phi + j, i * n_phi + jn
    c, d = (i + 1) * n_phi + j, (i + 1) * n_phi + jn
    tris = np.stack([np.stack([a, b, c], -1), np.stack([b, d, c], -1)], axis=2).reshape(-1, 3)
    return vertices, tris.astype(np.int32)


def _mesh_torus(center: np.ndarray, R: float, a: float, n_u: int, n_v: int) -> Tuple[np.ndarray, np.ndarray]:
    u = np.linspace(0.0, 2.0 * np.pi, n_u, endpoint=False)
    v = np.linspace(0.0, 2.0 * np.pi, n_v, endpoint=False)
    uu, vv = np.meshgrid(u, v, indexing="ij")
    cu, su, cv, sv = np.cos(uu), np.sin(uu), np.cos(vv), np.sin(vv)
    vertices = np.stack([(R + a * cv) * cu + center[0], (R + a * cv) * su + center[1], a * sv + center[2]],
                        axis=-1).reshape(-1, 3)
    i, j = np.meshgrid(np.arange(n_u), np.arange(n_v), indexing="ij")
    inext, jnext = (i + 1) % n_u, (j + 1) % n_v
    A, B = i * n_v + j, i * n_v + jnext
    C, D = inext * n_v + j, inext * n_v + jnext
    tris = np.stack([np.stack([A, B, C], -1), np.stack([B, D, C], -1)], axis=2).reshape(-1, 3)
    return vertices, tris.astype(np.int32)


def torus_mesh(R: float = 1.0, a: float = 0.35, n_u: int = 500, n_v: int = 200, center=(0.0, 0.0, 0.0),
               conductor_id: int = 0) -> TriMesh:
    """The reference's tensor-grid torus with an explicit grid (2 n_u n_v panels)."""
    v, t = _mesh_torus(np.asarray(center, float), float(R), float(a), int(n_u), int(n_v))
    return _finish(v, t, np.full(t.shape[0], conductor_id, np.int32))


def icosphere(subdivisions: int = 4, radius: float = 1.0, center=(0.0, 0.0, 0.0), conductor_id: int = 0) -> TriMesh:
    phi = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, phi, 0), (1, phi, 0), (-1, -phi, 0), (1, -phi, 0), (0, -1, phi), (0, 1, phi), (0, -1, -phi),
             (0, 1, -phi), (phi, 0, -1), (phi, 0, 1), (-phi, 0, -1), (-phi, 0, 1)]
    V = [np.asarray(p, float) / np.linalg.norm(p) for p in verts]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    for _ in range(int(subdivisions)):
        cache: Dict[Tuple[int, int], int] = {}

        def midpoint(i: int, j: int) -> int:
            key = (i, j) if i < j else (j, i)
            if key not in cache:
                m = V[i] + V[j]
                V.append(m / np.linalg.norm(m))
                cache[key] = len(V) - 1
            return cache[key]

        nf = []
        for a, b, c in F:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = nf
    vertices = np.asarray(V) * float(radius) + np.asarray(center, float)[None, :]
    tris = np.asarray(F, dtype=np.int32)
    return _finish(vertices, tris, np.full(tris.shape[0], conductor_id, np.int32))


def _cget(c: Any, key: str, default=None):
    return c.get(key, default) if isinstance(c, dict) else getattr(c, key, default)


def conductor_grids(spec: Any, target_h: float = 0.1) -> List[Tuple[str, tuple, int]]:
    """The tensor grid of every conductor of ``spec`` at ``target_h``, as
    (kind, generator arguments, conductor id) with the sizing rules of
    bem_mesh.py:27-136; kind is "plane" (z, L, n), "sphere" (center, radius,
    n_theta, n_phi) or "torus" (center, R, a, n_u, n_v)."""
    conductors = list(_cget(spec, "conductors", []) or [])
    charges = list(_cget(spec, "charges", []) or [])
    out: List[Tuple[str, tuple, int]] = []
    for idx, c in enumerate(conductors):
        typ = _cget(c, "type")
        cid = int(_cget(c, "id", idx))
        if typ == "plane":
            z = float(_cget(c, "z", 0.0))
            dmin = 0.3
            for ch in charges:
                if _cget(ch, "type") == "point":
                    dmin = max(dmin, abs(float(_cget(ch, "pos")[2] - z)))
            scale = float(os.getenv("EDE_BEM_PLANE_PATCH_SCALE", "1.0"))
            L = scale * max(8.0, 16.0 * dmin)
            out.append(("plane", (z, L, max(8, int(L / max(1e-3, target_h)))), cid))
        elif typ == "sphere":
            center = np.asarray(_cget(c, "center", [0.0, 0.0, 0.0]), float)
            radius = float(_cget(c, "radius", 1.0))
            base = max(1e-3, target_h)
            ds = max(1.0, float(os.getenv("EDE_BEM_SPHERE_DENSITY_SCALE", "1.5")))
            n_theta = max(10, int(np.ceil(ds * np.pi * radius / base)))
            n_phi = max(20, int(np.ceil(ds * 2.0 * np.pi * radius / base)))
            out.append(("sphere", (center, radius, n_theta, n_phi), cid))
        elif typ in ("torus", "toroid"):
            center = np.asarray(_cget(c, "center", [0.0, 0.0, 0.0]), float)
            R = float(_cget(c, "major_radius", _cget(c, "radius", 1.0)))
            a = float(_cget(c, "minor_radius", 0.25 * R))
            base = max(1e-3, target_h)
            ms = float(os.getenv("EDE_BEM_TORUS_MAJOR_SCALE", "1.0"))
            ns = float(os.getenv("EDE_BEM_TORUS_MINOR_SCALE", "1.0"))
            out.append(("torus", (center, R, a, max(24, int(np.ceil(ms * 2.0 * np.pi * R / base))),
                                  max(16, int(np.ceil(ns * 2.0 * np.pi * a / base)))), cid))
        else:
            raise NotImplementedError(f"Unsupported conductor type: {typ}")
    return out


_GENERATORS = {"plane": _mesh_plane_patch, "sphere": _mesh_sphere, "torus": _mesh_torus}


def generate_mesh(spec: Any, target_h: float = 0.1, logger: Optional[Any] = None) -> TriMesh:
    """Mesh every conductor of ``spec`` (same rules as bem_mesh.py:27-136)."""
    V_list: List[np.ndarray] = []
    T_list: List[np.ndarray] = []
    C_list: List[np.ndarray] = []
    offset = 0
    for kind, args, cid in conductor_grids(spec, target_h):
        v, t = _GENERATORS[kind](*args)
        V_list.append(v)
        T_list.append(t + offset)
        C_list.append(np.full(t.shape[0], cid, np.int32))
        offset += v.shape[0]
    if not V_list:
        return TriMesh(np.empty((0, 3)), np.empty((0, 3), np.int32), np.empty((0, 3)), np.empty((0, 3)), np.empty(0),
                       np.empty(0, np.int32))
    return _finish(np.vstack(V_list), np.vstack(T_list), np.concatenate(C_list))


__all__ = ["TriMesh", "conductor_grids", "generate_mesh", "icosphere", "torus_mesh"]
