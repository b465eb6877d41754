"""Graph-capturable single-layer operators for the device GMRES.

Each operator owns its output (and scratch) buffers, launches only on the
current stream and allocates nothing per call, so ``gmres_restart`` can
capture a whole restart cycle of ``A(v)`` + Arnoldi kernels in one CUDA
graph.  ``capturable = True`` advertises that.
"""
from __future__ import annotations

from typing import Optional

import torch
from torch import Tensor

from .. import _lib
from ..utils.config import K_E


class DenseOperator:
    """A(sigma) = dense single-layer operator (bem_kernel.py:157-230) on the GPU."""

    capturable = True

    def __init__(self, centroids: Tensor, areas: Tensor, self_integrals: Optional[Tensor] = None, *,
                 dtype: torch.dtype = torch.float64, device=None, k_e: float = K_E):
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.device, self.dtype, self.k_e = dev, dtype, float(k_e)
        self.c = centroids.to(dev, dtype).contiguous()
        self.a = areas.to(dev, dtype).contiguous()
        self.si = None if self_integrals is None else self_integrals.to(dev, dtype).contiguous()
        self.n = int(self.a.shape[0])
        L = _lib.load_library()
        nbytes = int(L.edfmm_dense_workspace_bytes(self.n, _lib.dtype_code(dtype)))
        self.ws = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=dev)
        self.nbytes = nbytes
        self.out = torch.empty(self.n, dtype=dtype, device=dev)

    def __call__(self, sigma: Tensor, out: Optional[Tensor] = None) -> Tensor:
        L = _lib.load_library()
        o = self.out if out is None else out
        s = sigma if sigma.is_contiguous() else sigma.contiguous()
        _lib.check(L.edfmm_dense_matvec_ws(_lib.ptr(self.c), _lib.ptr(s), _lib.ptr(self.a), _lib.ptr(self.si), self.n,
                                           _lib.dtype_code(self.dtype), self.k_e, _lib.ptr(o), _lib.ptr(self.ws),
                                           self.nbytes, _lib.stream_handle(self.device)), "edfmm_dense_matvec_ws")
        return o


class FmmOperator:
    """A(sigma) = FMM single-layer operator (LaplaceFmm3D.matvec) on a device plan."""

    capturable = True

    def __init__(self, plan: _lib.Plan, areas: Tensor, self_integrals: Optional[Tensor] = None, *,
                 k_e: float = K_E, flags: int = 0):
        self.plan = plan
        self.device, self.dtype = plan.device, plan.dtype
        self.a = areas.to(self.device, self.dtype).contiguous()
        self.si = None if self_integrals is None else self_integrals.to(self.device, self.dtype).contiguous()
        self.k_e = float(k_e)
        self.flags = int(flags)
        self.n = int(plan.info.n_points)
        self.out = torch.empty(self.n, dtype=self.dtype, device=self.device)
        # a first application builds the plan's lazily prepared tables outside
        # any capture: an FP32 plan's extreme-pair rows, and the transposed M2L
        # lists of the reference pair order.  FP64 plans prepare nothing lazily
        # (two-float mode builds its extreme rows when it is set), and an FP64
        # application is expensive (445 ms for the 5.6M-panel batched plan).
        if self.dtype == torch.float32 or self.flags != 0:
            self(torch.zeros(self.n, dtype=self.dtype, device=self.device))
            torch.cuda.synchronize(self.device)

    def __call__(self, sigma: Tensor, out: Optional[Tensor] = None) -> Tensor:
        o = self.out if out is None else out
        s = sigma if sigma.is_contiguous() else sigma.contiguous()
        return self.plan.matvec(s, self.a, self.si, k_e=self.k_e, out=o, flags=self.flags)

    def graph_state(self) -> tuple:
        """What a captured graph of this operator depends on besides its
        buffers: the plan's arithmetic (two-float mode launches other kernels)
        and its launch shapes."""
        return (getattr(self.plan, "arithmetic", "native"), tuple(sorted(self.plan.get_launch().items())))

    def set_active_mask(self, flags: Optional[Tensor], stride: int = 1) -> bool:
        """Batched plans: later applications skip the far-field rows and
        near-field leaves of instances with flags[k * stride] == 0 (their
        output rows are then unspecified); None removes the mask.  Returns
        False when the plan holds a single instance."""
        if self.plan.n_instances <= 1:
            return False
        self.plan.set_instance_mask(flags, stride)
        return True


__all__ = ["DenseOperator", "FmmOperator"]
