"""GPU singular / near-singular panel quadrature (libedfmm near-field module).

* :func:`self_integrals` -- the reference's per-panel self terms
  (core/bem.py:1781-1805) for every panel in one launch.
* :class:`NearCorrection` -- near pairs + correction weights
  (core/bem.py:475-667) built once per mesh and applied per matvec
  (core/bem.py:675-734).
* :func:`apply_near_quadrature_matvec_cuda` -- the reference CUDA module's
  on-the-fly entry point (core/bem_near_cuda.py:175-290).
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Tuple

import numpy as np
import torch
from torch import Tensor

from .. import _lib
from ..utils.config import K_E


def _dev64(x, device) -> Tensor:
    return torch.as_tensor(np.asarray(x) if not isinstance(x, Tensor) else x, dtype=torch.float64).to(device).contiguous()


def self_integrals(panel_vertices, centroids, *, order: int = 2, depth: int = 3, k_e: float = K_E,
                   device=None) -> Tensor:
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    L = _lib.load_library()
    pv = _dev64(panel_vertices, dev).reshape(-1, 9)
    c = _dev64(centroids, dev).reshape(-1, 3)
    out = torch.empty(c.shape[0], dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        _lib.check(L.edfmm_self_integrals(_lib.ptr(pv), _lib.ptr(c), c.shape[0], int(order), int(depth), float(k_e),
                                          _lib.ptr(out), _lib.stream_handle(dev)), "edfmm_self_integrals")
    return out


class NearCorrection:
    """Near pairs 0 < |C_i - C_j| <= f (R_i + R_j) and their quadrature weights."""

    def __init__(self, centroids, areas, panel_vertices, *, distance_factor: float = 1.5, order: int = 2,
                 depth: int = 3, k_e: float = K_E, dtype: torch.dtype = torch.float64, device=None):
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.device, self.dtype = dev, dtype
        L = _lib.load_library()
        self._L = L
        c = _dev64(centroids, dev).reshape(-1, 3)
        a = _dev64(areas, dev).reshape(-1)
        pv = _dev64(panel_vertices, dev).reshape(-1, 9)
        self.n = int(c.shape[0])
        h = C.c_void_p()
        with torch.cuda.device(dev):
            _lib.check(L.edfmm_near_create(_lib.ptr(c), _lib.ptr(a), _lib.ptr(pv), self.n, float(distance_factor),
                                           int(order), int(depth), float(k_e), _lib.dtype_code(dtype),
                                           _lib.stream_handle(dev), C.byref(h)), "edfmm_near_create")
        self._h = h
        self.n_pairs = int(L.edfmm_near_num_pairs(h))

    def astype(self, dtype: torch.dtype) -> "NearCorrection":
        """The same pairs and FP64 weights for a solve in ``dtype`` (no new
        pair search or quadrature; equal to building it with that dtype)."""
        if dtype == self.dtype:
            return self
        out = NearCorrection.__new__(NearCorrection)
        out.device, out.dtype, out._L, out.n, out.n_pairs = self.device, dtype, self._L, self.n, self.n_pairs
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self._L.edfmm_near_convert(self._h, _lib.dtype_code(dtype), _lib.stream_handle(self.device),
                                                  C.byref(h)), "edfmm_near_convert")
        out._h = h
        return out

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.edfmm_near_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def export(self):
        pairs = torch.empty(self.n_pairs, 2, dtype=torch.int64, device=self.device)
        w = torch.empty(self.n_pairs, dtype=torch.float64, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self._L.edfmm_near_export(self._h, _lib.ptr(pairs), _lib.ptr(w), _lib.stream_handle(self.device)),
                       "edfmm_near_export")
        return pairs, w

    def rows(self):
        ro, co = C.c_void_p(), C.c_void_p()
        _lib.check(self._L.edfmm_near_rows(self._h, C.byref(ro), C.byref(co)), "edfmm_near_rows")
        return ro, co

    def apply(self, sigma: Tensor, v_in: Optional[Tensor], out: Tensor) -> Tensor:
        """out = v_in + sum_j sigma_j delta_ij (out may be v_in)."""
        with torch.cuda.device(self.device):
            _lib.check(self._L.edfmm_near_apply(self._h, _lib.ptr(sigma), _lib.ptr(v_in), _lib.ptr(out),
                                                _lib.stream_handle(self.device)), "edfmm_near_apply")
        return out


# rows by target of the last few pair tensors passed to
# apply_near_quadrature_matvec_cuda: (tensor, its version counter, n, device,
# (row_off, cols)); the tensor is held, so its storage cannot be reused
# under a cached entry
_PAIR_ROWS: List[Tuple[Tensor, int, int, torch.device, Tuple[Tensor, Tensor]]] = []


def _pair_rows(near_pairs, n: int, dev: torch.device) -> Tuple[Tensor, Tensor]:
    """CSR rows by target (row_off int32 (n+1), cols int32, sources ascending
    within a row) of a (P, 2) (i, j) pair list."""
    if isinstance(near_pairs, Tensor):
        for t, ver, nn, d, rows in _PAIR_ROWS:
            if t is near_pairs and ver == near_pairs._version and nn == n and d == dev:
                return rows
    pr = torch.as_tensor(near_pairs).to(dev, torch.int64).reshape(-1, 2)
    if pr.shape[0]:
        pr = pr[torch.argsort(pr[:, 0] * n + pr[:, 1], stable=True)]  # (i, j) lexicographic
        counts = torch.bincount(pr[:, 0], minlength=n)
        row_off = torch.cat([counts.new_zeros(1), torch.cumsum(counts, 0)]).to(torch.int32)
        cols = pr[:, 1].to(torch.int32).contiguous()
    else:
        row_off = torch.zeros(n + 1, dtype=torch.int32, device=dev)
        cols = torch.zeros(1, dtype=torch.int32, device=dev)
    if isinstance(near_pairs, Tensor):
        _PAIR_ROWS.append((near_pairs, near_pairs._version, n, dev, (row_off, cols)))
        del _PAIR_ROWS[:-4]
    return row_off, cols


def apply_near_quadrature_matvec_cuda(V_far: Tensor, sigma: Tensor, *, centroids: Tensor, areas: Tensor,
                                      panel_vertices: Tensor, near_pairs, quad_order: int = 2,
                                      K_E: Optional[float] = None) -> Tensor:
    """The reference module's call (bem_near_cuda.py:175-290) on CUDA tensors.

    ``near_pairs`` is a (P, 2) (i, j) array or tensor (the reference passes
    them in any order); they are grouped into rows by target on the device,
    once per pair tensor: a solve that passes the same tensor every matvec
    reuses the rows (a tensor changed in place is regrouped).
    """
    from ..utils.config import K_E as _KE

    ke = float(_KE if K_E is None else K_E)
    L = _lib.load_library()
    dev, dt = V_far.device, V_far.dtype
    n = int(V_far.shape[0])
    row_off, cols = _pair_rows(near_pairs, n, dev)
    T = lambda x: x.to(dev, dt).contiguous()
    out = torch.empty_like(V_far)
    with torch.cuda.device(dev):
        _lib.check(L.edfmm_near_quadrature_matvec(_lib.ptr(T(V_far)), _lib.ptr(T(sigma)), _lib.ptr(T(centroids)),
                                                  _lib.ptr(T(areas)), _lib.ptr(T(panel_vertices).reshape(-1, 9)),
                                                  _lib.ptr(row_off), _lib.ptr(cols), n, ke, int(quad_order),
                                                  _lib.dtype_code(dt), _lib.ptr(out), _lib.stream_handle(dev)),
                   "edfmm_near_quadrature_matvec")
    return out


def point_charge_potential(points: Tensor, charges, *, k_e: float = K_E) -> Tensor:
    """sum_k k_e q_k / max(|x - r_k|, 1e-12) at CUDA points (core/bem.py:291-320)."""
    L = _lib.load_library()
    dev, dt = points.device, points.dtype
    ch = np.asarray([[float(q), *map(float, pos)] for q, pos in charges], dtype=np.float64).reshape(-1, 4)
    chd = torch.as_tensor(ch, device=dev) if ch.size else torch.zeros(1, 4, dtype=torch.float64, device=dev)
    out = torch.empty(points.shape[0], dtype=dt, device=dev)
    with torch.cuda.device(dev):
        _lib.check(L.edfmm_point_charge_potential(_lib.ptr(points.contiguous()), points.shape[0], _lib.ptr(chd),
                                                  ch.shape[0], float(k_e), _lib.dtype_code(dt), _lib.ptr(out),
                                                  _lib.stream_handle(dev)), "edfmm_point_charge_potential")
    return out


def potential_at_targets(targets: Tensor, centroids: Tensor, sigma: Tensor, areas: Tensor, *,
                         k_e: float = K_E) -> Tensor:
    """Induced potential of panel charges at targets (bem_potential_targets, bem_kernel.py:233-270)."""
    L = _lib.load_library()
    dev, dt = sigma.device, sigma.dtype
    T = lambda x: x.to(dev, dt).contiguous()
    t = T(targets)
    out = torch.empty(t.shape[0], dtype=dt, device=dev)
    with torch.cuda.device(dev):
        _lib.check(L.edfmm_dense_potential_targets(_lib.ptr(t), t.shape[0], _lib.ptr(T(centroids)), _lib.ptr(T(sigma)),
                                                   _lib.ptr(T(areas)), sigma.shape[0], _lib.dtype_code(dt), float(k_e),
                                                   _lib.ptr(out), _lib.stream_handle(dev)),
                   "edfmm_dense_potential_targets")
    return out


def field_at_targets(targets: Tensor, centroids: Tensor, sigma: Tensor, areas: Tensor, *,
                     k_e: float = K_E) -> Tensor:
    """Induced field of panel charges at targets, (M, 3) (bem_E_field_targets,
    bem_kernel.py:280-335: K_E sum_j sigma_j A_j (x - r_j) / max(r^2, 1e-24)^(3/2))."""
    L = _lib.load_library()
    dev, dt = sigma.device, sigma.dtype
    T = lambda x: x.to(dev, dt).contiguous()
    t = T(targets).reshape(-1, 3)
    out = torch.empty(t.shape[0], 3, dtype=dt, device=dev)
    with torch.cuda.device(dev):
        _lib.check(L.edfmm_dense_field_targets(_lib.ptr(t), t.shape[0], _lib.ptr(T(centroids)), _lib.ptr(T(sigma)),
                                               _lib.ptr(T(areas)), sigma.shape[0], _lib.dtype_code(dt), float(k_e),
                                               _lib.ptr(out), _lib.stream_handle(dev)),
                   "edfmm_dense_field_targets")
    return out


def near_potential_correction(V: Tensor, targets: Tensor, centroids: Tensor, areas: Tensor, sigma: Tensor,
                              panel_vertices: Tensor, *, distance_factor: float, quad_order: int = 2,
                              max_depth: Optional[int] = None, k_e: float = K_E) -> Tensor:
    """Target-side near-field quadrature (_apply_near_quadrature_potentials,
    bem.py:940-1046): returns V plus, for every panel j whose centroid is within
    distance_factor * sqrt(A_j / pi) of a target x, sigma_j (I_near(x) -
    K_E A_j / max(|C_j - x|, 1e-12)), with I_near the adaptive rule of panel j
    about x (depth ``max_depth``, 4 when None as for the reference's "telles").
    Computed in FP64 on the GPU; the result has V's dtype and device."""
    L = _lib.load_library()
    dev = V.device if V.is_cuda else torch.device("cuda", torch.cuda.current_device())
    D = lambda x: torch.as_tensor(x).to(dev, torch.float64).contiguous()
    t = D(targets).reshape(-1, 3)
    out = D(V).clone()
    depth = 4 if max_depth is None else int(max_depth)
    with torch.cuda.device(dev):
        _lib.check(L.edfmm_near_targets_correct(_lib.ptr(t), t.shape[0], _lib.ptr(D(centroids)), _lib.ptr(D(areas)),
                                                _lib.ptr(D(sigma)), _lib.ptr(D(panel_vertices)), int(areas.shape[0]),
                                                float(distance_factor), int(quad_order), depth, float(k_e),
                                                _lib.ptr(out), _lib.stream_handle(dev)),
                   "edfmm_near_targets_correct")
    return out.to(V.dtype).to(V.device)


def point_charge_field(points: Tensor, charges) -> Tensor:
    """Free-space field of point charges, sum_k K_E q_k (x - r_k) / max(|x - r_k|, 1e-12)^3
    (_free_space_E_field_at_points, bem.py:340-370), (M, 3) in the points' dtype."""
    P = points.reshape(-1, 3)
    E = torch.zeros_like(P)
    for q, pos in charges:
        R = P - torch.as_tensor(pos, dtype=P.dtype, device=P.device)[None, :]
        r = torch.linalg.norm(R, dim=1, keepdim=True).clamp_min(1e-12)
        E = E + (K_E * float(q)) * R / (r ** 3)
    return E


__all__ = ["self_integrals", "NearCorrection", "apply_near_quadrature_matvec_cuda", "point_charge_potential",
           "potential_at_targets", "field_at_targets", "point_charge_field", "near_potential_correction"]
