"""GPU FMM for the Laplace single-layer operator, mirroring ``electrodrive.fmm3d``."""
from .config import FmmConfig
from .bem_coupling import create_bem_fmm_backend
from .bem_fmm import LaplaceFmm3D, make_laplace_fmm_backend
from .interaction_lists import InteractionLists, build_interaction_lists
from .tree import FmmTree, build_fmm_tree

__all__ = [
    "FmmConfig",
    "create_bem_fmm_backend",
    "LaplaceFmm3D",
    "make_laplace_fmm_backend",
    "InteractionLists",
    "build_interaction_lists",
    "FmmTree",
    "build_fmm_tree",
]
