"""Conductor meshes generated on the GPU (no reference counterpart for the
device path; the meshes are the reference's, electrodrive/core/bem_mesh.py:27-212).

The host computes only the 1-D coordinate tables (numpy linspace values and
their sines and cosines, O(n_a + n_b) numbers); libedfmm's
``edfmm_mesh_grid`` forms every vertex and raw triangle of each conductor's
tensor grid on the device and ``edfmm_mesh_finish`` computes the panel
geometry (centroids, areas, unit normals) and drops degenerate panels, in
numpy's evaluation order, so a :class:`DeviceTriMesh` equals the host
generators' :class:`~electrodrive_gb300.core.bem_mesh.TriMesh` bit for bit.
Batched set-ups (many dimers) and training-data generation keep their meshes
on the device.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Any, Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch
from torch import Tensor

from .. import _lib
from .bem_mesh import TriMesh, conductor_grids


@dataclass
class DeviceTriMesh:
    """A TriMesh whose arrays live on the GPU (FP64 geometry, int32 indices)."""

    vertices: Tensor       # (n_vertices, 3)
    triangles: Tensor      # (n_panels, 3) int32
    centroids: Tensor      # (n_panels, 3)
    normals: Tensor        # (n_panels, 3)
    areas: Tensor          # (n_panels,)
    conductor_ids: Tensor  # (n_panels,) int32

    @property
    def n_panels(self) -> int:
        return int(self.triangles.shape[0])

    @property
    def panel_vertices(self) -> Tensor:
        return self.vertices[self.triangles.long()]

    def to_host(self) -> TriMesh:
        h = lambda t: t.cpu().numpy()
        return TriMesh(h(self.vertices), h(self.triangles), h(self.centroids), h(self.normals), h(self.areas),
                       h(self.conductor_ids))


def _tables(kind: str, args: tuple) -> Tuple[int, List[float], np.ndarray, np.ndarray]:
    """(libedfmm kind, parameters, table a, table b) of one grid, with the
    numpy calls of the host generators on their 1-D coordinate arrays."""
    if kind == "sphere":
        center, radius, n_theta, n_phi = args
        theta = np.linspace(0.0, np.pi, n_theta)
        phi = np.linspace(0.0, 2.0 * np.pi, n_phi, endpoint=False)
        ta = np.stack([np.sin(theta), np.cos(theta)], axis=1).ravel()
        tb = np.stack([np.sin(phi), np.cos(phi)], axis=1).ravel()
        c = np.asarray(center, float)
        return _lib.EDFMM_MESH_SPHERE, [c[0], c[1], c[2], float(radius), 0.0], ta, tb
    if kind == "torus":
        center, R, a, n_u, n_v = args
        u = np.linspace(0.0, 2.0 * np.pi, n_u, endpoint=False)
        v = np.linspace(0.0, 2.0 * np.pi, n_v, endpoint=False)
        ta = np.stack([np.sin(u), np.cos(u)], axis=1).ravel()
        tb = np.stack([np.sin(v), np.cos(v)], axis=1).ravel()
        c = np.asarray(center, float)
        return _lib.EDFMM_MESH_TORUS, [c[0], c[1], c[2], float(R), float(a)], ta, tb
    if kind == "plane":
        z, L, n = args
        x = np.linspace(-L / 2.0, L / 2.0, n + 1)
        y = np.linspace(-L / 2.0, L / 2.0, n + 1)
        return _lib.EDFMM_MESH_PLANE, [float(z), 0.0, 0.0, 0.0, 0.0], x, y
    raise NotImplementedError(f"Unsupported conductor type: {kind}")


def _grid_shape(kind: int, ta: np.ndarray, tb: np.ndarray) -> Tuple[int, int, int]:
    """(na, nb, raw triangles) of a grid."""
    if kind == _lib.EDFMM_MESH_PLANE:
        na, nb = ta.shape[0], tb.shape[0]
        return na, nb, 2 * (na - 1) * (nb - 1)
    na, nb = ta.shape[0] // 2, tb.shape[0] // 2
    return na, nb, 2 * (na - 1 if kind == _lib.EDFMM_MESH_SPHERE else na) * nb


def mesh_grids(grids: Sequence[Tuple[str, tuple, int]], device=None) -> DeviceTriMesh:
    """Mesh the (kind, arguments, conductor id) grids of :func:`conductor_grids`
    on the device: vertices back to back in grid order, the panels' geometry,
    degenerate panels removed (the host's _finish)."""
    L = _lib.load_library()
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    parts = [(_tables(kind, args), cid) for kind, args, cid in grids]
    shapes = [_grid_shape(k, ta, tb) for (k, _, ta, tb), _ in parts]
    nv = sum(na * nb for na, nb, _ in shapes)
    nt = sum(t for _, _, t in shapes)
    V = torch.empty(max(nv, 1), 3, dtype=torch.float64, device=dev)
    T = torch.empty(max(nt, 1), 3, dtype=torch.int32, device=dev)
    Cid = torch.empty(max(nt, 1), dtype=torch.int32, device=dev)
    with torch.cuda.device(dev):
        stream = _lib.stream_handle(dev)
        vo = to = 0
        keep = []
        for ((kind, params, ta, tb), cid), (na, nb, ntri) in zip(parts, shapes):
            tad = torch.as_tensor(ta, dtype=torch.float64).to(dev)
            tbd = torch.as_tensor(tb, dtype=torch.float64).to(dev)
            keep += [tad, tbd]
            par = (C.c_double * 5)(*params)
            _lib.check(L.edfmm_mesh_grid(kind, par, _lib.ptr(tad), na, _lib.ptr(tbd), nb, vo, int(cid),
                                         _lib.ptr(V[vo:]), _lib.ptr(T[to:]), _lib.ptr(Cid[to:]), stream),
                       "edfmm_mesh_grid")
            vo += na * nb
            to += ntri
        To = torch.empty(max(nt, 1), 3, dtype=torch.int32, device=dev)
        Co = torch.empty(max(nt, 1), dtype=torch.int32, device=dev)
        cen = torch.empty(max(nt, 1), 3, dtype=torch.float64, device=dev)
        nrm = torch.empty(max(nt, 1), 3, dtype=torch.float64, device=dev)
        ar = torch.empty(max(nt, 1), dtype=torch.float64, device=dev)
        n_out = C.c_int64(0)
        _lib.check(L.edfmm_mesh_finish(_lib.ptr(V), nv, _lib.ptr(T), _lib.ptr(Cid), nt, _lib.ptr(To), _lib.ptr(Co),
                                       _lib.ptr(cen), _lib.ptr(nrm), _lib.ptr(ar), C.byref(n_out), stream),
                   "edfmm_mesh_finish")
    m = int(n_out.value)
    return DeviceTriMesh(V[:nv], To[:m], cen[:m], nrm[:m], ar[:m], Co[:m])


def generate_mesh_device(spec: Any, target_h: float = 0.1, device=None) -> DeviceTriMesh:
    """generate_mesh (the reference's bem_mesh.py:27-136 sizing and
    generators) on the GPU."""
    return mesh_grids(conductor_grids(spec, target_h), device)


def torus_mesh_device(R: float = 1.0, a: float = 0.35, n_u: int = 500, n_v: int = 200, center=(0.0, 0.0, 0.0),
                      conductor_id: int = 0, device=None) -> DeviceTriMesh:
    """torus_mesh (2 n_u n_v panels) on the GPU."""
    return mesh_grids([("torus", (np.asarray(center, float), float(R), float(a), int(n_u), int(n_v)),
                        int(conductor_id))], device)


__all__ = ["DeviceTriMesh", "generate_mesh_device", "mesh_grids", "torus_mesh_device"]
