"""Near-field P2P on the GPU (electrodrive/fmm3d/kernels_gpu.py:51-274).

``apply_p2p_gpu`` evaluates the reference's near-field contribution
``q_s / max(|x_t - x_s|, eps)`` over the P2P leaf pairs, with the diagonal
removed only in the self leaf pair of a single tree (kernels_cpu.py:83-153,
kernels_gpu.py:170-190), in one launch of libedfmm's warp-per-leaf kernel.
With distinct source and target trees the pairs are the two-tree lists and
nothing is excluded.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any, Optional

import torch
from torch import Tensor

from .interaction_lists import InteractionLists
from .tree import FmmTree


@dataclass
class P2PResult:
    potential: Tensor
    n_pairs: int
    n_interactions: int


def apply_p2p_gpu(source_tree: FmmTree, target_tree: FmmTree, charges_src: Tensor, lists: InteractionLists, *,
                  cfg: Optional[Any] = None, logger: Optional[Any] = None, out: Optional[Tensor] = None) -> P2PResult:
    """charges_src in the source tree's order (as in the reference); returns
    potentials in the target tree's order."""
    if charges_src.shape[0] != source_tree.n_points:
        raise ValueError("charges_src length must equal source_tree.n_points "
                         f"(got {charges_src.shape[0]} vs {source_tree.n_points}).")
    if source_tree.dtype != charges_src.dtype:
        raise ValueError(f"charges_src.dtype ({charges_src.dtype}) must match source_tree.dtype ({source_tree.dtype}).")
    if lists.truncated:
        raise RuntimeError("apply_p2p_gpu: interaction lists were truncated")
    plan = source_tree.plan
    q = charges_src.to(plan.device).contiguous()
    if target_tree is not source_tree:
        from .. import _lib
        from .interaction_lists import two_tree_handle

        if target_tree.dtype != source_tree.dtype:
            raise ValueError(f"target_tree.dtype ({target_tree.dtype}) must match source_tree.dtype "
                             f"({source_tree.dtype}).")
        handle = two_tree_handle(source_tree, target_tree, lists, lists.mac_theta)
        plan.set_charges(source_tree.map_to_original_order(q).contiguous())
        phi = handle.stage(_lib.EDFMM_TARGETS_P2P)
        if out is not None:
            out.copy_(phi)
            phi = out
        return P2PResult(potential=phi, n_pairs=int(handle.n_p2p_pairs), n_interactions=int(handle.p2p_interactions))
    if abs(plan.info.mac_theta - lists.mac_theta) > 0:
        plan.rebuild_lists(lists.mac_theta)
    # the plan stores charges in tree order internally; it receives them in
    # original order, so undo the tree permutation first
    plan.set_charges(source_tree.map_to_original_order(q).contiguous())
    phi = plan.p2p()
    if out is not None:
        out.copy_(phi)
        phi = out
    return P2PResult(potential=phi, n_pairs=int(plan.info.n_p2p_pairs), n_interactions=int(plan.info.p2p_interactions))


apply_p2p_gpu_tiled = apply_p2p_gpu

__all__ = ["P2PResult", "apply_p2p_gpu", "apply_p2p_gpu_tiled"]
