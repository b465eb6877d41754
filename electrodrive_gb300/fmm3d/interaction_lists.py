"""Dual-tree interaction lists built on the GPU
(electrodrive/fmm3d/interaction_lists.py:374-629).

The pair sets and their (tgt, src) order are bit-identical to the
reference's.  Pairs are kept as (K, 2) int64 tensors on the GPU; the
reference's Python list views (``p2p_pairs``, ``u_list`` ...) are materialised
on first access only.  Lists between a source tree and a distinct target
tree hold a handle of libedfmm's two-tree evaluation object, through which
the tree-level P2P, M2L, L2L and L2P run between the two trees.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional, Tuple

import torch
from torch import Tensor

from .tree import FmmTree


@dataclass
class InteractionStats:
    num_p2p_pairs: int = 0
    num_m2l_pairs: int = 0
    num_stack_pops: int = 0
    max_stack_size: int = 0
    num_mac_accept: int = 0
    num_mac_reject: int = 0
    num_leaf_leaf: int = 0
    truncated: bool = False

    def as_dict(self) -> Dict[str, int | bool]:
        return dict(self.__dict__)


@dataclass
class InteractionLists:
    """Node-pair lists; ``p2p`` / ``m2l`` are (K, 2) (src, tgt) tensors sorted by (tgt, src)."""

    p2p: Tensor
    m2l: Tensor
    mac_theta: float
    n_nodes: int
    same_tree: bool = True
    truncated: bool = False
    stats: Optional[InteractionStats] = field(default=None, repr=False)
    _cache: dict = field(default_factory=dict, repr=False)
    # two-tree lists: libedfmm's evaluation object (source plan + copy of the
    # target tree + these lists + the target locals)
    targets: Optional[Any] = field(default=None, repr=False)
    source_tree: Optional[FmmTree] = field(default=None, repr=False)
    target_tree: Optional[FmmTree] = field(default=None, repr=False)

    @property
    def num_p2p_pairs(self) -> int:
        return int(self.p2p.shape[0])

    @property
    def num_m2l_pairs(self) -> int:
        return int(self.m2l.shape[0])

    def _pairs(self, key: str) -> List[Tuple[int, int]]:
        if key not in self._cache:
            t = self.p2p if key == "p2p" else self.m2l
            self._cache[key] = [tuple(x) for x in t.cpu().tolist()]
        return self._cache[key]

    @property
    def p2p_pairs(self) -> List[Tuple[int, int]]:
        return self._pairs("p2p")

    @property
    def m2l_pairs(self) -> List[Tuple[int, int]]:
        return self._pairs("m2l")

    def _per_target(self, key: str) -> List[List[int]]:
        ck = key + "_rows"
        if ck not in self._cache:
            rows: List[List[int]] = [[] for _ in range(self.n_nodes)]
            for s, t in self._pairs(key):
                rows[t].append(s)
            self._cache[ck] = rows
        return self._cache[ck]

    @property
    def u_list(self) -> List[List[int]]:
        return self._per_target("p2p")

    @property
    def v_list(self) -> List[List[int]]:
        return self._per_target("m2l")

    w_list = v_list
    x_list = v_list

    @property
    def u_self_mask(self) -> List[bool]:
        mask = [False] * self.n_nodes
        if self.same_tree:
            sel = self.p2p[self.p2p[:, 0] == self.p2p[:, 1], 1].cpu().tolist()
            for t in sel:
                mask[t] = True
        return mask

    def as_tensors(self, device: Optional[torch.device] = None) -> Tuple[Tensor, Tensor]:
        if device is None:
            return self.p2p, self.m2l
        return self.p2p.to(device), self.m2l.to(device)

    def to(self, device) -> "InteractionLists":
        self.p2p = self.p2p.to(device)
        self.m2l = self.m2l.to(device)
        return self


def build_interaction_lists(source_tree: FmmTree, target_tree: Optional[FmmTree] = None, mac_theta: float = 0.5, *,
                            max_pairs: Optional[int] = None, sort_pairs: bool = True) -> InteractionLists:
    """Classify node pairs into P2P (near) and M2L (far) lists with the reference MAC.

    With ``target_tree`` None or the source tree itself, the same-tree lists
    of the operator; with a distinct target tree, the two-tree lists
    (sources = source-tree nodes, targets = target-tree nodes) of
    interaction_lists.py:531-577.  ``sort_pairs`` is accepted for signature
    compatibility (the output is always sorted by (tgt, src)).
    """
    if target_tree is None:
        target_tree = source_tree
    if mac_theta <= 0.0:
        raise ValueError("mac_theta must be positive")
    if mac_theta >= 1.0:
        raise ValueError("mac_theta should be < 1.0 for a meaningful MAC")
    if target_tree is not source_tree:
        return _build_two_tree_lists(source_tree, target_tree, float(mac_theta), max_pairs)
    plan = source_tree.plan
    plan.rebuild_lists(float(mac_theta))
    p2p, m2l = plan.export_lists()
    total = p2p.shape[0] + m2l.shape[0]
    if max_pairs is not None and total > max_pairs:
        raise RuntimeError("Interaction list truncated-MAC is likely misconfigured or pair count exploded.")
    stats = InteractionStats(num_p2p_pairs=int(p2p.shape[0]), num_m2l_pairs=int(m2l.shape[0]))
    return InteractionLists(p2p=p2p, m2l=m2l, mac_theta=float(mac_theta), n_nodes=source_tree.n_nodes,
                            same_tree=True, stats=stats)


def _build_two_tree_lists(source_tree: FmmTree, target_tree: FmmTree, mac_theta: float,
                          max_pairs: Optional[int]) -> InteractionLists:
    from .. import _lib

    if source_tree.device != target_tree.device:
        raise ValueError("source and target trees must be on the same device")
    if source_tree.dtype != target_tree.dtype:
        raise ValueError(f"source and target trees must share a dtype ({source_tree.dtype} vs {target_tree.dtype})")
    handle = _lib.Targets.from_plan(source_tree.plan, target_tree.plan, mac_theta)
    p2p, m2l = handle.export_lists()
    if max_pairs is not None and p2p.shape[0] + m2l.shape[0] > max_pairs:
        raise RuntimeError("Interaction list truncated-MAC is likely misconfigured or pair count exploded.")
    stats = InteractionStats(num_p2p_pairs=int(p2p.shape[0]), num_m2l_pairs=int(m2l.shape[0]))
    return InteractionLists(p2p=p2p, m2l=m2l, mac_theta=mac_theta, n_nodes=target_tree.n_nodes, same_tree=False,
                            stats=stats, targets=handle, source_tree=source_tree, target_tree=target_tree)


def two_tree_handle(source_tree: FmmTree, target_tree: FmmTree, lists: Optional[InteractionLists],
                    mac_theta: float) -> Any:
    """The two-tree evaluation object for (source_tree, target_tree): the one
    ``lists`` carries when it was built for these trees at the source plan's
    current expansion order, else a fresh one."""
    if (lists is not None and lists.targets is not None and lists.source_tree is source_tree
            and lists.target_tree is target_tree
            and lists.targets.order == int(source_tree.plan.info.expansion_order)):
        return lists.targets
    theta = lists.mac_theta if lists is not None else mac_theta
    fresh = _build_two_tree_lists(source_tree, target_tree, float(theta), None)
    if lists is not None and lists.targets is not None:
        lists.targets = fresh.targets
    return fresh.targets


def verify_interaction_lists(source_tree: FmmTree, target_tree: FmmTree, lists: InteractionLists) -> None:
    """Structural checks of interaction_lists.py:580-622 on the tensors."""
    ns, nt = source_tree.n_nodes, target_tree.n_nodes
    for t in (lists.p2p, lists.m2l):
        if t.numel():
            assert int(t[:, 0].min()) >= 0 and int(t[:, 0].max()) < ns, "source index out of range"
            assert int(t[:, 1].min()) >= 0 and int(t[:, 1].max()) < nt, "target index out of range"
    if lists.p2p.numel():
        assert bool(source_tree.node_is_leaf[lists.p2p[:, 0]].all()
                    and target_tree.node_is_leaf[lists.p2p[:, 1]].all()), "p2p pair with a non-leaf node"


__all__ = ["InteractionStats", "InteractionLists", "build_interaction_lists", "two_tree_handle",
           "verify_interaction_lists"]
