"""Legacy BEM/FMM bridge (electrodrive/fmm3d/bem_coupling.py:24-142).

``create_bem_fmm_backend(cfg).apply(src_centroids, sigma, areas, self_integrals=...)``
builds the GPU FMM for the given geometry on each call (as the reference
does) and returns ``K_E * sum_j sigma_j A_j / r_ij (+ self term)``.
"""
from __future__ import annotations

from typing import Any, Optional

import torch
from torch import Tensor

from .bem_fmm import LaplaceFmm3D
from .config import FmmConfig


class FmmBemBackend:
    def __init__(self, cfg: FmmConfig, logger: Optional[Any] = None) -> None:
        self.cfg = cfg
        self.logger = logger

    def apply(self, src_centroids: Tensor, sigma: Tensor, areas: Optional[Tensor] = None, *,
              self_integrals: Optional[Tensor] = None) -> Tensor:
        if src_centroids.ndim != 2 or src_centroids.shape[1] != 3:
            raise ValueError("src_centroids must have shape (N, 3)")
        n = src_centroids.shape[0]
        if sigma.shape != (n,):
            raise ValueError("sigma must have shape (N,)")
        if areas is None:
            areas = torch.ones(n, dtype=src_centroids.dtype)
        c = src_centroids.detach().cpu().contiguous()
        a = areas.detach().cpu().to(c.dtype).contiguous()
        fmm = LaplaceFmm3D(c, a, max_leaf_size=self.cfg.leaf_size, theta=self.cfg.mac_theta,
                           expansion_order=self.cfg.expansion_order, logger=self.logger)
        si = None if self_integrals is None else self_integrals.to(sigma.device, c.dtype)
        return fmm.matvec(sigma=sigma.to(c.dtype), src_centroids=c, areas=a, tile_size=1024, self_integrals=si)


def create_bem_fmm_backend(cfg: Optional[FmmConfig] = None, logger: Optional[Any] = None) -> FmmBemBackend:
    return FmmBemBackend(cfg or FmmConfig(), logger)


__all__ = ["FmmBemBackend", "create_bem_fmm_backend"]
