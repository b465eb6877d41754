"""FMM configuration, field-compatible with electrodrive/fmm3d/config.py:31-171."""
from __future__ import annotations

from dataclasses import dataclass
from typing import Literal, Optional

import torch

BackendKind = Literal["cpu", "gpu", "auto"]
PrecisionKind = Literal["single", "double", "mixed"]

FMM_L_MAX_HARD_LIMIT = 32
FMM_M2L_LMAX_FACTOR = 2
# Orders this implementation supports (register-resident M2L up to 8, a
# shared-memory M2L kernel for 9-10).
FMM_MAX_SUPPORTED_ORDER = 10


@dataclass
class FmmConfig:
    """Same fields, defaults and validation as the reference ``FmmConfig``.

    ``precision`` selects the expansion dtype exactly as the reference does
    (config.py:146-156): "double" -> float64, "single"/"mixed" -> float32.
    """

    kernel: str = "laplace_single_layer"
    expansion_order: int = 8
    mac_theta: float = 0.5
    leaf_size: int = 64
    backend: BackendKind = "auto"
    precision: PrecisionKind = "mixed"
    use_fft_m2l: bool = True
    use_gpu: bool = True
    use_multi_gpu: bool = False
    use_mpi: bool = False
    dtype: Optional[torch.dtype] = None
    p2p_batch_size: Optional[int] = None

    def __post_init__(self) -> None:
        if self.dtype is None:
            self.dtype = torch.float64 if self.precision == "double" else torch.float32
        self.validate()

    def validate(self) -> None:
        if self.expansion_order <= 0:
            raise ValueError("expansion_order must be positive")
        if not (0.1 <= self.mac_theta <= 0.9):
            raise ValueError("mac_theta should be in [0.1, 0.9] for stability")
        if self.leaf_size <= 0:
            raise ValueError("leaf_size must be positive")
        l_max_m2l = FMM_M2L_LMAX_FACTOR * self.expansion_order
        if l_max_m2l > FMM_L_MAX_HARD_LIMIT:
            raise ValueError(
                "expansion_order too large for current spherical-harmonics backend: M2L uses "
                f"l_max={l_max_m2l} (factor {FMM_M2L_LMAX_FACTOR}x p) but "
                f"FMM_L_MAX_HARD_LIMIT={FMM_L_MAX_HARD_LIMIT}."
            )
        if self.dtype not in (torch.float32, torch.float64):
            raise ValueError(f"dtype must be torch.float32 or torch.float64; got {self.dtype!r}")
        if self.p2p_batch_size is not None and self.p2p_batch_size <= 0:
            raise ValueError("p2p_batch_size must be positive if specified")


__all__ = ["FMM_L_MAX_HARD_LIMIT", "FMM_M2L_LMAX_FACTOR", "FMM_MAX_SUPPORTED_ORDER", "FmmConfig", "BackendKind",
           "PrecisionKind"]
