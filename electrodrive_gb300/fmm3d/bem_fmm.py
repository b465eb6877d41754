"""GPU FMM backend for the Laplace single-layer BEM operator
(electrodrive/fmm3d/bem_fmm.py:104-940).

``make_laplace_fmm_backend(...).matvec(...)`` keeps the reference's
signatures, argument checks and error types.  The octree, interaction lists
and every FMM stage run in libedfmm on the GPU; there is no CPU execution
path.  A CPU ``sigma`` is copied to the device (through pinned staging
buffers) and the result copied back, exactly as the reference's GPU backend
returns results on sigma's device.
"""
from __future__ import annotations

from typing import Any, Optional

import torch
from torch import Tensor

from .. import _lib
from ..utils.config import K_E
from .config import FMM_MAX_SUPPORTED_ORDER, BackendKind, FmmConfig
from .interaction_lists import InteractionLists, build_interaction_lists
from .tree import FmmTree, build_fmm_tree


class LaplaceFmm3D:
    """GPU Laplace FMM for V_i = sum_j K_E sigma_j A_j / |c_i - c_j| (+ self term)."""

    def __init__(self, src_centroids: Tensor, areas: Tensor, *, max_leaf_size: int = 64, theta: float = 0.5,
                 use_dipole: bool = True, logger: Optional[Any] = None, expansion_order: Optional[int] = None,
                 backend: BackendKind = "auto", device: Optional[torch.device | str] = None,
                 reference_pair_order: bool = False) -> None:
        if src_centroids.ndim != 2 or src_centroids.shape[1] != 3:
            raise ValueError("src_centroids must have shape (N, 3)")
        if areas.ndim != 1 or areas.shape[0] != src_centroids.shape[0]:
            raise ValueError("areas must have shape (N,) matching src_centroids")
        if src_centroids.device.type != "cpu" or areas.device.type != "cpu":
            raise ValueError("LaplaceFmm3D currently supports only CPU tensors for src_centroids and areas.")
        self.src_centroids = src_centroids
        self.areas = areas
        self.N = int(src_centroids.shape[0])
        self.max_leaf_size = int(max_leaf_size)
        self.theta = float(theta)
        self.use_dipole = bool(use_dipole)
        self.logger = logger
        self.device = src_centroids.device
        self.dtype = src_centroids.dtype
        self.reference_pair_order = bool(reference_pair_order)
        cfg_kwargs = dict(mac_theta=self.theta, leaf_size=self.max_leaf_size, dtype=self.dtype, backend=backend)
        if expansion_order is not None:
            cfg_kwargs["expansion_order"] = int(expansion_order)
        self.cfg = FmmConfig(**cfg_kwargs)
        if self.cfg.expansion_order > FMM_MAX_SUPPORTED_ORDER:
            raise ValueError(f"expansion_order {self.cfg.expansion_order} > {FMM_MAX_SUPPORTED_ORDER} is not supported")
        if backend == "cpu":
            raise ValueError("electrodrive_gb300 runs the FMM on the GPU only; use backend='gpu' or 'auto'")
        if not torch.cuda.is_available() or not self.cfg.use_gpu:
            raise RuntimeError("GPU backend requested but CUDA/use_gpu not available.")
        self.backend = "gpu"
        self.fmm_device = torch.device(device or "cuda")
        if self.fmm_device.index is None:
            self.fmm_device = torch.device("cuda", torch.cuda.current_device())
        self.cfg.backend = "gpu"
        _lib.load_library()
        pts = src_centroids.to(self.fmm_device).contiguous()
        self.tree: FmmTree = build_fmm_tree(pts, leaf_size=int(self.cfg.leaf_size), mac_theta=self.cfg.mac_theta)
        self.tree_gpu = self.tree
        self.tree_cpu = self.tree
        self._plan = self.tree.plan
        self._plan.set_order(int(self.cfg.expansion_order))
        self.lists: Optional[InteractionLists] = None
        self._areas_gpu = areas.to(self.fmm_device, dtype=self.dtype).contiguous()
        self._pinned = {}

    # ------------------------------------------------------------------ info
    @property
    def plan(self) -> _lib.Plan:
        return self._plan

    @property
    def n_p2p_pairs(self) -> int:
        return int(self._plan.info.n_p2p_pairs)

    @property
    def n_m2l_pairs(self) -> int:
        return int(self._plan.info.n_m2l_pairs)

    def interaction_lists(self) -> InteractionLists:
        if self.lists is None:
            self.lists = build_interaction_lists(self.tree, self.tree, mac_theta=self.cfg.mac_theta)
        return self.lists

    # ----------------------------------------------------------------- checks
    def _check_geometry_consistency(self, src_centroids: Tensor, areas: Tensor) -> None:
        if src_centroids.data_ptr() != self.src_centroids.data_ptr():
            raise ValueError("LaplaceFmm3D.matvec called with different src_centroids than the ones used to build "
                             "the FMM tree.")
        if areas.data_ptr() != self.areas.data_ptr():
            raise ValueError("LaplaceFmm3D.matvec called with different areas than the ones used to build the FMM tree.")
        if src_centroids.device.type != "cpu" or areas.device.type != "cpu":
            raise ValueError("LaplaceFmm3D currently requires matvec geometry tensors to live on the CPU.")
        if src_centroids.dtype != self.dtype or areas.dtype != self.dtype:
            raise ValueError(f"LaplaceFmm3D geometry dtype mismatch: expected {self.dtype}, got "
                             f"{src_centroids.dtype} / {areas.dtype}.")

    def _staging(self, name: str) -> Tensor:
        buf = self._pinned.get(name)
        if buf is None:
            buf = torch.empty(self.N, dtype=self.dtype, pin_memory=True)
            self._pinned[name] = buf
        return buf

    # ----------------------------------------------------------------- matvec
    def matvec(self, *, sigma: Tensor, src_centroids: Tensor, areas: Tensor, tile_size: int,
               self_integrals: Optional[Tensor], logger: Optional[Any] = None, kernel: Optional[Any] = None,
               **kwargs) -> Tensor:
        """External matvec compatible with ``bem_matvec_gpu(backend="external")``."""
        self._check_geometry_consistency(src_centroids, areas)
        if kernel is not None and type(kernel).__name__ not in ("LaplaceSingleLayerKernel",):
            raise ValueError("LaplaceFmm3D currently only supports LaplaceSingleLayerKernel.")
        N = int(sigma.shape[0])
        if N != self.N:
            raise ValueError(f"sigma has length {N}, but FMM backend was built for {self.N} panels.")
        sdev = sigma.device
        if sdev.type == "cuda":
            if sdev != self.fmm_device:
                raise ValueError(f"LaplaceFmm3D.matvec CUDA sigma must live on {self.fmm_device}, got {sdev}.")
        elif sdev.type != "cpu":
            raise ValueError("LaplaceFmm3D.matvec only supports CPU or CUDA sigma.")
        if sigma.dtype != self.dtype:
            raise ValueError(f"LaplaceFmm3D sigma dtype mismatch: expected {self.dtype}, got {sigma.dtype}.")
        if self_integrals is not None:
            if self_integrals.shape != sigma.shape:
                raise ValueError("self_integrals must have shape (N,) matching sigma.")
            if self_integrals.device != sdev:
                raise ValueError("self_integrals must be on the same device as sigma "
                                 f"(sigma={sdev}, self_integrals={self_integrals.device}).")
            if self_integrals.dtype != sigma.dtype:
                raise ValueError("self_integrals must have the same dtype as sigma "
                                 f"(sigma={sigma.dtype}, self_integrals={self_integrals.dtype}).")
        if N == 0:
            return torch.zeros_like(sigma)
        flags = _lib.EDFMM_REFERENCE_PAIR_ORDER if self.reference_pair_order else 0
        if sdev.type == "cuda":
            s = sigma.contiguous()
            si = self_integrals.contiguous() if self_integrals is not None else None
            return self._plan.matvec(s, self._areas_gpu, si, k_e=float(K_E), flags=flags)
        # host sigma: pinned staging, async copies on the current stream
        h_sig = self._staging("sigma")
        h_sig.copy_(sigma)
        d_sig = h_sig.to(self.fmm_device, non_blocking=True)
        d_si = None
        if self_integrals is not None:
            h_si = self._staging("self")
            h_si.copy_(self_integrals)
            d_si = h_si.to(self.fmm_device, non_blocking=True)
        d_out = self._plan.matvec(d_sig, self._areas_gpu, d_si, k_e=float(K_E), flags=flags)
        h_out = self._staging("out")
        h_out.copy_(d_out, non_blocking=True)
        torch.cuda.current_stream(self.fmm_device).synchronize()
        return h_out.clone()


def make_laplace_fmm_backend(src_centroids: Tensor, areas: Tensor, *, max_leaf_size: int = 64, theta: float = 0.5,
                             use_dipole: bool = True, logger: Optional[Any] = None,
                             expansion_order: Optional[int] = None, backend: BackendKind = "auto",
                             device: Optional[torch.device | str] = None, **kwargs) -> LaplaceFmm3D:
    """Convenience constructor (bem_fmm.py:888-940)."""
    return LaplaceFmm3D(src_centroids=src_centroids, areas=areas, max_leaf_size=max_leaf_size, theta=theta,
                        use_dipole=use_dipole, logger=logger, expansion_order=expansion_order, backend=backend,
                        device=device, **kwargs)


__all__ = ["LaplaceFmm3D", "make_laplace_fmm_backend"]
