"""Physical constants and solver configuration (electrodrive/utils/config.py:34-153)."""
from __future__ import annotations

import math
from dataclasses import dataclass

EPS_0 = 8.854187817e-12
K_E = 1.0 / (4.0 * math.pi * EPS_0)


@dataclass
class BEMConfig:
    """The reference BEMConfig's fields and defaults (utils/config.py:78-153)."""

    use_gpu: bool = True
    fp64: bool = False
    initial_h: float = 0.2
    max_refine_passes: int = 3
    target_bc_inf_norm: float = 1e-7
    linear_tol_factor: float = 0.1
    gmres_tol: float = 5e-8
    gmres_maxiter: int = 2000
    gmres_restart: int = 256
    gmres_log_every: int = 10
    vram_autotune: bool = True
    target_vram_fraction: float = 0.95
    vram_cap_gb: float = 24.0
    target_peak_gb: float = 20.0
    min_tile: int = 1024
    max_tile: int = 1 << 18
    tile_size: int = 0
    tile_mem_divisor: float = 2.0
    use_near_quadrature: bool = False
    use_near_quadrature_matvec: bool = False
    near_quadrature_distance_factor: float = 1.5
    near_quadrature_order: int = 2
    use_precond: bool = True
