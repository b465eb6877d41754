"""Physical constants and solver configuration (electrodrive/utils/config.py:34-153)."""
from __future__ import annotations

import math
from dataclasses import dataclass

EPS_0 = 8.854187817e-12
K_E = 1.0 / (4.0 * math.pi * EPS_0)


@dataclass
class BEMConfig:
    """Subset of the reference BEMConfig (utils/config.py:78-153) used by the solve path."""

    fp64: bool = False
    gmres_restart: int = 256
    gmres_tol: float = 5e-8
    gmres_maxiter: int = 2000
    use_near_quadrature: bool = False
    use_near_quadrature_matvec: bool = False
    near_quadrature_order: int = 2
    near_quadrature_distance_factor: float = 1.5
    tile_mem_divisor: float = 2.5
    target_vram_fraction: float = 0.9
