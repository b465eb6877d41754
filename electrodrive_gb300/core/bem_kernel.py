"""Single-layer BEM operator entry point (electrodrive/core/bem_kernel.py:558-707).

``bem_matvec_gpu`` keeps the reference's signature and backend names:
``"external"`` calls ``matvec_impl`` (e.g. ``LaplaceFmm3D.matvec``) with the
reference's keyword arguments; ``"auto"``, ``"torch_tiled"`` and ``"keops"``
all run libedfmm's dense CUDA operator (``edfmm_dense_matvec``).  Results are
returned on sigma's device.
"""
from __future__ import annotations

import os
from typing import Any, Callable, Optional

import torch
from torch import Tensor

from .. import _lib
from ..utils.config import K_E


class LaplaceSingleLayerKernel:
    """G(r) = K_E / r (the only kernel the reference's fast paths implement)."""

    name = "laplace_single_layer"

    def potential(self, diff: Tensor, r: Tensor) -> Tensor:
        return K_E / r


DEFAULT_SINGLE_LAYER_KERNEL = LaplaceSingleLayerKernel()


def _ensure_tile_size(tile_size: Optional[int]) -> int:
    if tile_size is not None and tile_size > 0:
        return int(tile_size)
    env_val = os.getenv("EDE_BEM_TILE_SIZE")
    if env_val is not None:
        try:
            v = int(env_val)
            if v > 0:
                return v
        except ValueError:
            pass
    return 1024


def _dense(sigma: Tensor, src_centroids: Tensor, areas: Tensor, self_integrals: Optional[Tensor]) -> Tensor:
    dev = sigma.device if sigma.is_cuda else torch.device("cuda", torch.cuda.current_device())
    dt = sigma.dtype
    c = src_centroids.to(dev, dt).contiguous()
    a = areas.to(dev, dt).contiguous()
    s = sigma.to(dev).contiguous()
    si = None if self_integrals is None else self_integrals.to(dev, dt).contiguous()
    out = _lib.dense_matvec(c, s, a, si, k_e=float(K_E))
    return out if sigma.is_cuda else out.to(sigma.device)


def bem_matvec_gpu(sigma: Tensor, src_centroids: Tensor, areas: Tensor, *, tile_size: int = 1024,
                   self_integrals: Optional[Tensor] = None, logger: Optional[Any] = None, use_keops: bool = False,
                   kernel: Optional[Any] = None, backend: str = "auto", matvec_impl: Optional[Callable[..., Tensor]] = None,
                   **kwargs) -> Tensor:
    """Matrix-free V = sum_j K_ij sigma_j A_j with K_ii = self_integrals_i (or 0)."""
    if "self_correction" in kwargs and self_integrals is None:
        self_integrals = kwargs.get("self_correction")
    if backend not in {"auto", "torch_tiled", "keops", "external"}:
        raise ValueError(f"Unknown BEM backend: {backend!r}")
    ker = kernel or DEFAULT_SINGLE_LAYER_KERNEL
    tile_size = _ensure_tile_size(tile_size)
    if backend == "external":
        if matvec_impl is None:
            raise ValueError("backend='external' requires matvec_impl.")
        return matvec_impl(sigma=sigma, src_centroids=src_centroids, areas=areas, tile_size=tile_size,
                           self_integrals=self_integrals, logger=logger, kernel=ker, **kwargs)
    if not isinstance(ker, LaplaceSingleLayerKernel):
        raise ValueError("electrodrive_gb300 implements the Laplace single-layer kernel only")
    n = int(sigma.shape[0])
    if n == 0:
        return torch.zeros_like(sigma)
    return _dense(sigma, src_centroids, areas, self_integrals)


def bem_potential_targets(targets: Tensor, src_centroids: Tensor, areas: Tensor, sigma: Tensor, *,
                          tile_size: int = 1024, method: str = "auto", fmm_threshold: int = 20000,
                          leaf_size: int = 64, expansion_order: int = 8, mac_theta: float = 0.5) -> Tensor:
    """Induced potential K_E sum_j sigma_j A_j / |x - c_j| at targets
    (electrodrive/core/bem_kernel.py:233-335).  ``method`` "dense" is the
    reference's direct sum (r^2 clamped at 1e-24); "fmm" builds a plan of the
    panels and a target tree (distances clamped at the dtype's epsilon);
    "auto" takes the FMM when panels x targets exceeds fmm_threshold^2."""
    from ..utils.config import K_E
    from .bem_near import potential_at_targets

    _ensure_tile_size(tile_size)
    if targets.ndim != 2 or targets.shape[-1] != 3:
        raise ValueError("targets must have shape (M, 3)")
    n, m = int(sigma.shape[0]), int(targets.shape[0])
    if method not in ("auto", "dense", "fmm"):
        raise ValueError(f"unknown method {method!r}")
    use_fmm = method == "fmm" or (method == "auto" and n * m > fmm_threshold * fmm_threshold)
    if not use_fmm:
        return potential_at_targets(targets, src_centroids, sigma, areas)
    dev = sigma.device if sigma.is_cuda else torch.device("cuda", torch.cuda.current_device())
    dt = sigma.dtype
    plan = _lib.Plan(src_centroids.to(dev, dt).contiguous(), leaf_size=leaf_size, mac_theta=mac_theta,
                     expansion_order=expansion_order)
    tg = plan.targets(targets.to(dev, dt))
    return tg.potential(sigma.to(dev, dt), areas.to(dev, dt), k_e=K_E)


def bem_E_field_targets(targets: Tensor, src_centroids: Tensor, areas: Tensor, sigma: Tensor, tile_size: int = 1024,
                        *, logger: Optional[Any] = None, use_keops: bool = False, kernel: Optional[Any] = None,
                        backend: str = "auto", method: str = "dense", leaf_size: int = 64, expansion_order: int = 8,
                        mac_theta: float = 0.5) -> Tensor:
    """Induced field at targets, (M, 3) (electrodrive/core/bem_kernel.py:914):
    K_E sum_j sigma_j A_j (x - r_j) / max(|x - r_j|^2, 1e-24)^(3/2), the
    reference's Laplace fast path, evaluated on the GPU.  ``backend`` accepts
    the reference's names ("auto", "torch_tiled", "keops"); all run the same
    dense kernel.  ``method="fmm"`` (not in the reference) evaluates the field
    by FMM instead: a plan of the panels, a target tree, near sums over the
    P2P lists and minus the gradient of the local expansions (distances within
    the dtype's epsilon contribute nothing).  Only the Laplace kernel is
    supported."""
    from .bem_near import field_at_targets

    if backend not in {"auto", "torch_tiled", "keops"}:
        raise ValueError(f"Unknown backend for bem_E_field_targets: {backend!r}")
    if method not in ("dense", "fmm"):
        raise ValueError(f"unknown method {method!r}")
    if kernel is not None and not isinstance(kernel, LaplaceSingleLayerKernel):
        raise ValueError("only the Laplace single-layer kernel is supported")
    _ensure_tile_size(tile_size)
    if targets.ndim != 2 or targets.shape[-1] != 3:
        raise ValueError("targets must have shape (M, 3)")
    if int(sigma.shape[0]) == 0 or int(targets.shape[0]) == 0:
        return torch.zeros(int(targets.shape[0]), 3, dtype=sigma.dtype, device=sigma.device)
    if method == "dense":
        return field_at_targets(targets, src_centroids, sigma, areas)
    dev = sigma.device if sigma.is_cuda else torch.device("cuda", torch.cuda.current_device())
    dt = sigma.dtype
    plan = _lib.Plan(src_centroids.to(dev, dt).contiguous(), leaf_size=leaf_size, mac_theta=mac_theta,
                     expansion_order=expansion_order)
    tg = plan.targets(targets.to(dev, dt))
    return tg.field(sigma.to(dev, dt), areas.to(dev, dt), k_e=K_E)


__all__ = ["LaplaceSingleLayerKernel", "DEFAULT_SINGLE_LAYER_KERNEL", "bem_matvec_gpu", "bem_potential_targets",
           "bem_E_field_targets"]
