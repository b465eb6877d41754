"""Tree-level FMM stages on the GPU (electrodrive/fmm3d/multipole_operators.py:1520-1765).

``p2m -> m2m -> m2l -> l2l -> l2p`` mirror the reference's tree drivers but
operate on the expansion buffers of the tree's device plan.  The expansions
are analytic complex solid harmonics (Condon-Shortley phase) scaled per node
by its radius, not the reference's least-squares proxy fits; they agree with
the reference in the potential they produce, not coefficient by coefficient.
With distinct source and target trees, ``m2l`` fills the target tree's locals
(held by the two-tree evaluation object of the interaction lists) and
``l2l`` / ``l2p`` on those locals run in the target tree.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any, Optional

import torch
from torch import Tensor

from .. import _lib
from .config import FmmConfig
from .interaction_lists import InteractionLists
from .tree import FmmTree


@dataclass
class MultipoleCoefficients:
    """Handle to the plan's multipole buffer (``data`` materialises it)."""

    tree: FmmTree
    charges: Tensor  # tree order

    @property
    def data(self) -> Tensor:
        return self.tree.plan.expansions()[0]


@dataclass
class LocalCoefficients:
    tree: FmmTree
    # two-tree evaluation object when the locals belong to a target tree
    targets: Optional[Any] = None

    @property
    def data(self) -> Tensor:
        if self.targets is not None:
            return self.targets.stage(_lib.EDFMM_TARGETS_LOCALS)
        return self.tree.plan.expansions()[1]


class MultipoleOpStats:
    def __init__(self) -> None:
        self.p2m_calls = self.m2m_calls = self.m2l_calls = self.l2l_calls = self.l2p_calls = 0
        self.extras: dict = {}

    def as_dict(self) -> dict:
        return dict(p2m_calls=self.p2m_calls, m2m_calls=self.m2m_calls, m2l_calls=self.m2l_calls,
                    l2l_calls=self.l2l_calls, l2p_calls=self.l2p_calls, **self.extras)


def _prepare(tree: FmmTree, cfg: FmmConfig) -> _lib.Plan:
    plan = tree.plan
    if plan.info.expansion_order != cfg.expansion_order:
        plan.set_order(int(cfg.expansion_order))
    if plan.info.mac_theta != cfg.mac_theta:
        plan.rebuild_lists(float(cfg.mac_theta))
    return plan


def p2m(tree: FmmTree, charges: Tensor, cfg: FmmConfig, stats: Optional[MultipoleOpStats] = None):
    """charges in ORIGINAL point order (as the reference's tree driver takes them)."""
    plan = _prepare(tree, cfg)
    q = charges.to(device=plan.device, dtype=plan.dtype).contiguous()
    plan.set_charges(q)
    plan.stage("p2m")
    if stats is not None:
        stats.p2m_calls += int(tree.node_is_leaf.sum())
    return MultipoleCoefficients(tree=tree, charges=tree.map_to_tree_order(q))


def m2m(tree: FmmTree, multipoles: MultipoleCoefficients, cfg: FmmConfig, stats: Optional[MultipoleOpStats] = None):
    _prepare(tree, cfg).stage("m2m")
    if stats is not None:
        stats.m2m_calls += max(tree.n_nodes - 1, 0)
    return multipoles


def m2l(source_tree: FmmTree, target_tree: FmmTree, multipoles: MultipoleCoefficients, cfg: FmmConfig,
        stats: Optional[MultipoleOpStats] = None, lists: Optional[InteractionLists] = None,
        reference_pair_order: bool = False):
    if target_tree is not source_tree:
        # source -> target translation over the two-tree M2L list (the pairs
        # are applied as listed, (src, tgt); the reference's swapped unpacking,
        # multipole_operators.py:1671, has no meaning between two trees)
        from .interaction_lists import two_tree_handle

        if lists is not None and lists.truncated:
            raise RuntimeError("FMM M2L interaction lists were truncated. Increase max_pairs or relax mac_theta so "
                               "that all far-field pairs are represented.")
        _prepare(source_tree, cfg)
        handle = two_tree_handle(source_tree, target_tree, lists, float(cfg.mac_theta))
        handle.stage(_lib.EDFMM_TARGETS_M2L)
        if stats is not None:
            stats.m2l_calls += int(handle.n_m2l_pairs)
        return LocalCoefficients(tree=target_tree, targets=handle)
    plan = _prepare(source_tree, cfg)
    if lists is not None and plan.info.mac_theta != lists.mac_theta:
        plan.rebuild_lists(lists.mac_theta)
    flags = _lib.EDFMM_REFERENCE_PAIR_ORDER if reference_pair_order else 0
    plan.stage("m2l", flags)
    if stats is not None:
        stats.m2l_calls += int(plan.info.n_m2l_pairs)
    return LocalCoefficients(tree=source_tree)


def l2l(tree: FmmTree, locals_: LocalCoefficients, cfg: FmmConfig, stats: Optional[MultipoleOpStats] = None):
    if locals_.targets is not None:
        if locals_.tree is not tree:
            raise ValueError("l2l: locals_ belong to another tree")
        locals_.targets.stage(_lib.EDFMM_TARGETS_L2L)
        if stats is not None:
            stats.l2l_calls += max(tree.n_nodes - 1, 0)
        return locals_
    _prepare(tree, cfg).stage("l2l")
    if stats is not None:
        stats.l2l_calls += max(tree.n_nodes - 1, 0)
    return locals_


def l2p(tree: FmmTree, locals_: LocalCoefficients, cfg: FmmConfig, stats: Optional[MultipoleOpStats] = None) -> Tensor:
    """Far-field potential at the tree points, TREE order, pure 1/r kernel."""
    if locals_.targets is not None:
        if locals_.tree is not tree:
            raise ValueError("l2p: locals_ belong to another tree")
        out = locals_.targets.stage(_lib.EDFMM_TARGETS_L2P)
        if stats is not None:
            stats.l2p_calls += int(tree.node_is_leaf.sum())
        return out
    out = _prepare(tree, cfg).l2p()
    if stats is not None:
        stats.l2p_calls += int(tree.node_is_leaf.sum())
    return out


__all__ = ["MultipoleCoefficients", "LocalCoefficients", "MultipoleOpStats", "p2m", "m2m", "m2l", "l2l", "l2p"]
