"""Adaptive octree built on the GPU (electrodrive/fmm3d/tree.py:170-1050).

``build_fmm_tree`` returns an :class:`FmmTree` whose SoA arrays
(``node_centers``, ``node_half_extents``, ``node_radii``, ``node_levels``,
``node_parents``, ``node_children``, ``node_ranges``, ``node_is_leaf``,
``index_map``) are bit-identical to the reference builder's for the same
points.  Unlike the reference, the build runs on the GPU (points may be given
on the CPU or on a CUDA device); the tree's tensors live on the CUDA device.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Tuple

import torch
from torch import Tensor

from .. import _lib


@dataclass
class TreeNode:
    """Object view of one node (tree.py:60-110); built on demand."""

    index: int
    parent: Optional[int]
    level: int
    center: Tensor
    half_extent: Tensor
    start: int
    end: int
    children: Tuple[Optional[int], ...]

    @property
    def is_leaf(self) -> bool:
        return all(c is None for c in self.children)

    @property
    def n_points(self) -> int:
        return self.end - self.start

    @property
    def half_size(self) -> Tensor:
        return self.half_extent


@dataclass
class TreeStatistics:
    n_points: int
    n_nodes: int
    n_leaves: int
    max_depth: int
    nodes_per_level: Tensor
    leaf_size_min: int
    leaf_size_max: int
    leaf_size_mean: float


@dataclass
class BoundingBox:
    center: Tensor
    half_extent: Tensor


class FmmTree:
    """Octree SoA on the GPU plus the plan that owns the device data."""

    def __init__(self, plan: _lib.Plan, points_tree: Tensor, soa: dict, leaf_size: int, max_depth: int):
        self._plan = plan
        self.points = points_tree
        self.index_map = soa["index_map"]
        self.inverse_index_map = torch.empty_like(self.index_map)
        if self.index_map.numel() > 0:
            self.inverse_index_map[self.index_map] = torch.arange(
                self.index_map.shape[0], device=self.index_map.device, dtype=self.index_map.dtype)
        self.node_centers = soa["node_centers"]
        self.node_half_extents = soa["node_half_extents"]
        self.node_radii = soa["node_radii"]
        self.node_levels = soa["node_levels"]
        self.node_parents = soa["node_parents"]
        self.node_children = soa["node_children"]
        self.node_ranges = soa["node_ranges"]
        self.node_is_leaf = soa["node_is_leaf"]
        self.leaf_size = int(leaf_size)
        self.max_depth = int(max_depth)
        if self.node_centers.shape[0] > 0:
            pts = self.points
            mn, mx = pts.min(dim=0).values, pts.max(dim=0).values
            self.global_bbox = BoundingBox(center=0.5 * (mn + mx), half_extent=torch.clamp(0.5 * (mx - mn), min=0.0))
        else:
            z = torch.zeros(3, dtype=self.points.dtype, device=self.points.device)
            self.global_bbox = BoundingBox(center=z, half_extent=z.clone())
        self._nodes: Optional[List[TreeNode]] = None

    # -------------------------------------------------------------- basics
    @property
    def plan(self) -> _lib.Plan:
        return self._plan

    @property
    def device(self) -> torch.device:
        return self.points.device

    @property
    def dtype(self) -> torch.dtype:
        return self.points.dtype

    @property
    def n_points(self) -> int:
        return int(self.points.shape[0])

    @property
    def n_nodes(self) -> int:
        return int(self.node_levels.shape[0])

    @property
    def root(self) -> int:
        return 0 if self.n_nodes > 0 else -1

    @property
    def depth_warnings(self) -> int:
        return int(self._plan.info.depth_warnings)

    @property
    def tree_to_original(self) -> Tensor:
        return self.index_map

    @property
    def original_to_tree(self) -> Tensor:
        return self.inverse_index_map

    @property
    def nodes(self) -> List[TreeNode]:
        """TreeNode objects (copied to the host on first use)."""
        if self._nodes is None:
            c = self.node_centers.cpu()
            h = self.node_half_extents.cpu()
            par = self.node_parents.cpu().tolist()
            ch = self.node_children.cpu().tolist()
            rg = self.node_ranges.cpu().tolist()
            lv = self.node_levels.cpu().tolist()
            self._nodes = [
                TreeNode(index=i, parent=None if par[i] < 0 else par[i], level=lv[i], center=c[i], half_extent=h[i],
                         start=rg[i][0], end=rg[i][1], children=tuple(None if x < 0 else x for x in ch[i]))
                for i in range(self.n_nodes)
            ]
        return self._nodes

    def leaf_indices(self) -> Tensor:
        return torch.nonzero(self.node_is_leaf, as_tuple=False).view(-1).to(torch.int64)

    def leaves(self) -> List[TreeNode]:
        return [self.nodes[int(i)] for i in self.leaf_indices().tolist()]

    def map_to_tree_order(self, values: Tensor) -> Tensor:
        if values.shape[0] != self.n_points:
            raise ValueError(f"values.shape[0] = {values.shape[0]} does not match n_points = {self.n_points}")
        if self.index_map.numel() == 0:
            return values
        return values[self.index_map.to(values.device)]

    def map_to_original_order(self, values: Tensor) -> Tensor:
        if values.shape[0] != self.n_points:
            raise ValueError(f"values.shape[0] = {values.shape[0]} does not match n_points = {self.n_points}")
        if self.index_map.numel() == 0:
            return values
        return values[self.inverse_index_map.to(values.device)]

    map_from_tree_order = map_to_original_order

    def statistics(self) -> TreeStatistics:
        if self.n_nodes == 0:
            return TreeStatistics(self.n_points, 0, 0, -1, torch.empty(0, dtype=torch.int64), 0, 0, 0.0)
        levels = self.node_levels.to(torch.int64)
        max_depth = int(levels.max().item())
        nodes_per_level = torch.bincount(levels, minlength=max_depth + 1)
        leaf_idx = self.leaf_indices()
        sizes = (self.node_ranges[leaf_idx, 1] - self.node_ranges[leaf_idx, 0]).to(torch.int64)
        return TreeStatistics(self.n_points, self.n_nodes, int(leaf_idx.numel()), max_depth, nodes_per_level,
                              int(sizes.min().item()), int(sizes.max().item()), float(sizes.float().mean().item()))

    def describe(self) -> str:
        st = self.statistics()
        lines = [f"FmmTree: n_points={st.n_points}, n_nodes={st.n_nodes}, n_leaves={st.n_leaves}, "
                 f"max_depth={st.max_depth}",
                 f"  leaf_size: min={st.leaf_size_min}, max={st.leaf_size_max}, mean={st.leaf_size_mean:.2f}"]
        if st.nodes_per_level.numel() > 0:
            lines.append("  nodes_per_level: " + ", ".join(
                f"{lvl}:{int(c)}" for lvl, c in enumerate(st.nodes_per_level.tolist())))
        return "\n".join(lines)

    def to(self, device, dtype: Optional[torch.dtype] = None) -> "FmmTree":
        """Move the SoA views (the device plan stays where it was built)."""
        device = torch.device(device)
        dt = self.dtype if dtype is None else dtype
        for name in ("points", "node_centers", "node_half_extents", "node_radii"):
            setattr(self, name, getattr(self, name).to(device=device, dtype=dt))
        for name in ("index_map", "inverse_index_map", "node_levels", "node_parents", "node_children",
                     "node_ranges", "node_is_leaf"):
            setattr(self, name, getattr(self, name).to(device=device))
        self.global_bbox = BoundingBox(self.global_bbox.center.to(device=device, dtype=dt),
                                       self.global_bbox.half_extent.to(device=device, dtype=dt))
        return self


def build_fmm_tree(points: Tensor, *, leaf_size: int = 64, max_depth: int = 32, mac_theta: float = 0.5,
                   device: Optional[torch.device] = None) -> FmmTree:
    """Build the adaptive octree of ``points`` (N, 3) on the GPU.

    Same arguments and validation as the reference (tree.py:968-1050); the
    CPU-only restriction is lifted.  ``mac_theta`` pre-builds the interaction
    lists of the same plan (``build_interaction_lists`` rebuilds them if asked
    for another value).
    """
    if max_depth <= 0:
        raise ValueError(f"max_depth must be positive, got {max_depth}")
    if max_depth > 64:
        raise ValueError(f"max_depth={max_depth} is too large (limit 64)")
    if leaf_size <= 0:
        raise ValueError(f"leaf_size must be positive, got {leaf_size}")
    if points.ndim != 2 or points.shape[-1] != 3:
        raise ValueError(f"points must have shape (N, 3), got {tuple(points.shape)}")
    if not torch.is_floating_point(points):
        raise TypeError(f"points must be floating point, got {points.dtype}")
    _lib.load_library()
    dev = torch.device(device) if device is not None else (
        points.device if points.is_cuda else torch.device("cuda", torch.cuda.current_device()))
    pts = points.to(device=dev).contiguous()
    plan = _lib.Plan(pts, leaf_size=leaf_size, max_depth=max_depth, mac_theta=mac_theta, expansion_order=8)
    soa = plan.export_tree()
    points_tree = pts[soa["index_map"]] if pts.shape[0] > 0 else pts
    tree = FmmTree(plan, points_tree, soa, leaf_size, max_depth)
    if plan.info.depth_warnings:
        import warnings

        warnings.warn(
            f"max_depth={max_depth} reached in {plan.info.depth_warnings} node(s) with more than "
            f"leaf_size={leaf_size} points; consider revisiting tree parameters or discretisation.",
            RuntimeWarning,
        )
    return tree


__all__ = ["TreeNode", "TreeStatistics", "FmmTree", "BoundingBox", "build_fmm_tree"]
