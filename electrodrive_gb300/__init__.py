"""GB300-native FMM-accelerated Laplace single-layer BEM operator.

The compute path is ``libedfmm.so`` (hand-written sm_103a CUDA behind the C
ABI of ``include/edfmm.h``); ``electrodrive_gb300.fmm3d`` mirrors the
reference's ``electrodrive.fmm3d`` entry points on top of it.
"""
from ._lib import EdfmmError, load_library

__version__ = "0.1.0"

__all__ = ["EdfmmError", "load_library", "__version__"]
