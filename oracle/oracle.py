"""ctypes front end of the CPU oracle (oracle/edfmm_oracle.c).

TEST INFRASTRUCTURE ONLY.  tests/, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` leg of ``bench.py`` use this module as the checker; the
product package ``electrodrive_gb300`` never imports it.

Every function mirrors a reference routine (paths inside the reference
project):

* :func:`build_tree`   -- ``electrodrive/fmm3d/tree.py:968`` (``build_fmm_tree``)
* :func:`build_lists`  -- ``electrodrive/fmm3d/interaction_lists.py:531``
* :func:`p2p`          -- ``electrodrive/fmm3d/kernels_cpu.py:183`` (FP64 accumulation)
* :func:`direct`       -- ``electrodrive/fmm3d/sanity_suite.py:83-121``
* :func:`dense_matvec` -- ``electrodrive/core/bem_kernel.py:157-230``
* :func:`fmm_matvec`   -- ``electrodrive/fmm3d/bem_fmm.py:460-594`` with analytic
  translation operators in FP64.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libedfmm_oracle.so")
_lib = None

K_E = 1.0 / (4.0 * np.pi * 8.854187817e-12)


def build() -> str:
    """Compile the oracle with its Makefile (gcc, no GPU needed)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
            os.path.join(_HERE, "edfmm_oracle.c")
        ):
            build()
        L = C.CDLL(_LIB_PATH)
        vp, i64, i32, dbl = C.c_void_p, C.c_int64, C.c_int, C.c_double
        L.orc_tree_build.restype = vp
        L.orc_tree_build.argtypes = [vp, i64, i32, i32, i32]
        L.orc_tree_n_nodes.restype = i64
        L.orc_tree_n_nodes.argtypes = [vp]
        L.orc_tree_n_depth_warnings.restype = i32
        L.orc_tree_n_depth_warnings.argtypes = [vp]
        L.orc_tree_export.argtypes = [vp] * 10
        L.orc_tree_free.argtypes = [vp]
        L.orc_lists_build.restype = vp
        L.orc_lists_build.argtypes = [vp, dbl]
        L.orc_lists_n_p2p.restype = i64
        L.orc_lists_n_p2p.argtypes = [vp]
        L.orc_lists_n_m2l.restype = i64
        L.orc_lists_n_m2l.argtypes = [vp]
        L.orc_lists_export.argtypes = [vp, vp, vp]
        L.orc_lists_free.argtypes = [vp]
        L.orc_p2p.argtypes = [vp, vp, i64, vp, vp, i64, dbl, vp]
        L.orc_direct.argtypes = [vp, vp, i64, vp, i64, vp]
        L.orc_dense_matvec.argtypes = [vp, vp, vp, vp, i64, dbl, vp]
        L.orc_fmm_matvec.restype = i32
        L.orc_fmm_matvec.argtypes = [vp, vp, vp, vp, vp, vp, i32, dbl, i32, dbl, vp, vp, vp]
        L.orc_num_threads.restype = i32
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


@dataclass
class OracleTree:
    """Reference SoA tree (tree.py:286-348) plus the oracle handle."""

    handle: int
    dtype: np.dtype
    points_tree: np.ndarray
    index_map: np.ndarray
    node_centers: np.ndarray
    node_half_extents: np.ndarray
    node_radii: np.ndarray
    node_levels: np.ndarray
    node_parents: np.ndarray
    node_children: np.ndarray
    node_ranges: np.ndarray
    node_is_leaf: np.ndarray
    depth_warnings: int

    @property
    def n_nodes(self) -> int:
        return int(self.node_levels.shape[0])

    def free(self):
        if self.handle:
            lib().orc_tree_free(self.handle)
            self.handle = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def build_tree(points: np.ndarray, leaf_size: int = 64, max_depth: int = 32) -> OracleTree:
    pts = np.ascontiguousarray(points)
    if pts.dtype not in (np.float32, np.float64):
        raise TypeError("points must be float32 or float64")
    n = pts.shape[0]
    L = lib()
    h = L.orc_tree_build(_p(pts), n, int(pts.dtype == np.float64), int(leaf_size), int(max_depth))
    m = L.orc_tree_n_nodes(h)
    im = np.empty(n, np.int64)
    c = np.empty((m, 3), np.float64)
    he = np.empty((m, 3), np.float64)
    r = np.empty(m, np.float64)
    lv = np.empty(m, np.int32)
    par = np.empty(m, np.int64)
    ch = np.empty((m, 8), np.int64)
    rg = np.empty((m, 2), np.int64)
    lf = np.empty(m, np.uint8)
    L.orc_tree_export(h, _p(im), _p(c), _p(he), _p(r), _p(lv), _p(par), _p(ch), _p(rg), _p(lf))
    dt = pts.dtype
    return OracleTree(
        handle=h,
        dtype=dt,
        points_tree=pts[im] if n else pts,
        index_map=im,
        node_centers=c.astype(dt),
        node_half_extents=he.astype(dt),
        node_radii=r.astype(dt),
        node_levels=lv,
        node_parents=par,
        node_children=ch,
        node_ranges=rg,
        node_is_leaf=lf.astype(bool),
        depth_warnings=int(L.orc_tree_n_depth_warnings(h)),
    )


@dataclass
class OracleLists:
    handle: int
    p2p_pairs: np.ndarray  # (K, 2) (src, tgt) sorted by (tgt, src)
    m2l_pairs: np.ndarray

    def free(self):
        if self.handle:
            lib().orc_lists_free(self.handle)
            self.handle = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def build_lists(tree: OracleTree, mac_theta: float = 0.5) -> OracleLists:
    if not (0.0 < mac_theta < 1.0):
        raise ValueError("mac_theta must be in (0, 1)")
    L = lib()
    h = L.orc_lists_build(tree.handle, float(mac_theta))
    a = np.empty((L.orc_lists_n_p2p(h), 2), np.int64)
    b = np.empty((L.orc_lists_n_m2l(h), 2), np.int64)
    L.orc_lists_export(h, _p(a), _p(b))
    return OracleLists(handle=h, p2p_pairs=a, m2l_pairs=b)


def p2p(points_tree, charges_tree, node_ranges, p2p_pairs, eps) -> np.ndarray:
    pts = np.ascontiguousarray(points_tree, dtype=np.float64)
    q = np.ascontiguousarray(charges_tree, dtype=np.float64)
    rg = np.ascontiguousarray(node_ranges, dtype=np.int64)
    pr = np.ascontiguousarray(p2p_pairs, dtype=np.int64)
    out = np.empty(pts.shape[0], np.float64)
    lib().orc_p2p(_p(pts), _p(q), pts.shape[0], _p(rg), _p(pr), pr.shape[0], float(eps), _p(out))
    return out


def direct(points, charges, target_idx=None) -> np.ndarray:
    pts = np.ascontiguousarray(points, dtype=np.float64)
    q = np.ascontiguousarray(charges, dtype=np.float64)
    n = pts.shape[0]
    idx = np.arange(n, dtype=np.int64) if target_idx is None else np.ascontiguousarray(target_idx, np.int64)
    out = np.empty(idx.shape[0], np.float64)
    lib().orc_direct(_p(pts), _p(q), n, _p(idx), idx.shape[0], _p(out))
    return out


def dense_matvec(centroids, sigma, areas, self_integrals=None, ke=K_E) -> np.ndarray:
    c = np.ascontiguousarray(centroids, dtype=np.float64)
    s = np.ascontiguousarray(sigma, dtype=np.float64)
    a = np.ascontiguousarray(areas, dtype=np.float64)
    si = None if self_integrals is None else np.ascontiguousarray(self_integrals, dtype=np.float64)
    out = np.empty(c.shape[0], np.float64)
    lib().orc_dense_matvec(_p(c), _p(s), _p(a), _p(si), c.shape[0], float(ke), _p(out))
    return out


def fmm_matvec(tree: OracleTree, lists: OracleLists, points, sigma, areas, self_integrals=None, *,
               p: int = 8, ke: float = K_E, reference_pair_order: bool = False, eps=None,
               return_parts: bool = False):
    pts = np.ascontiguousarray(points, dtype=np.float64)
    s = np.ascontiguousarray(sigma, dtype=np.float64)
    a = np.ascontiguousarray(areas, dtype=np.float64)
    si = None if self_integrals is None else np.ascontiguousarray(self_integrals, dtype=np.float64)
    n = pts.shape[0]
    if eps is None:
        eps = float(np.finfo(tree.dtype).eps)
    out = np.empty(n, np.float64)
    far = np.empty(n, np.float64)
    near = np.empty(n, np.float64)
    rc = lib().orc_fmm_matvec(tree.handle, lists.handle, _p(pts), _p(s), _p(a), _p(si), int(p), float(ke),
                              int(bool(reference_pair_order)), float(eps), _p(out), _p(far), _p(near))
    if rc != 0:
        raise ValueError(f"oracle fmm_matvec failed with status {rc}")
    if return_parts:
        return out, far, near
    return out


def num_threads() -> int:
    return int(lib().orc_num_threads())


def _declare_bem():
    L = lib()
    if getattr(L, "_bem_declared", False):
        return L
    vp, i64, i32, dbl = C.c_void_p, C.c_int64, C.c_int, C.c_double
    L.orc_self_integrals.argtypes = [vp, vp, i64, i32, i32, dbl, vp]
    L.orc_near_pairs.restype = i64
    L.orc_near_pairs.argtypes = [vp, vp, i64, dbl, vp, i64]
    L.orc_near_weights.argtypes = [vp, vp, vp, vp, i64, i32, i32, dbl, vp]
    L._bem_declared = True
    return L


def self_integrals(panel_vertices, centroids, order=2, depth=3, ke=K_E) -> np.ndarray:
    """near_singular_quadrature self terms (bem_quadrature.py:217-308, bem.py:1781-1805)."""
    L = _declare_bem()
    pv = np.ascontiguousarray(panel_vertices, dtype=np.float64)
    c = np.ascontiguousarray(centroids, dtype=np.float64)
    out = np.empty(c.shape[0])
    L.orc_self_integrals(_p(pv), _p(c), c.shape[0], int(order), int(depth), float(ke), _p(out))
    return out


def near_pairs(centroids, areas, factor=1.5) -> np.ndarray:
    """_build_near_pairs_for_panels (bem.py:475-555), O(N^2)."""
    L = _declare_bem()
    c = np.ascontiguousarray(centroids, dtype=np.float64)
    a = np.ascontiguousarray(areas, dtype=np.float64)
    n = L.orc_near_pairs(_p(c), _p(a), c.shape[0], float(factor), None, 0)
    out = np.empty((n, 2), np.int64)
    L.orc_near_pairs(_p(c), _p(a), c.shape[0], float(factor), _p(out), n)
    return out


def near_weights(centroids, areas, panel_vertices, pairs, order=2, depth=3, ke=K_E) -> np.ndarray:
    """_precompute_near_correction_weights (bem.py:558-667)."""
    L = _declare_bem()
    c = np.ascontiguousarray(centroids, dtype=np.float64)
    a = np.ascontiguousarray(areas, dtype=np.float64)
    pv = np.ascontiguousarray(panel_vertices, dtype=np.float64)
    pr = np.ascontiguousarray(pairs, dtype=np.int64)
    w = np.empty(pr.shape[0])
    L.orc_near_weights(_p(c), _p(a), _p(pv), _p(pr), pr.shape[0], int(order), int(depth), float(ke), _p(w))
    return w
