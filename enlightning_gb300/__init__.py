"""GB300-native (sm_103a) implementation of Enlightning's per-patch time advance.

The compute path is libenlightning_gpu.so (CUDA kernels behind the C-ABI in
include/enlightning_gpu.h).  This package holds its in-tree build, the ctypes
binding, and the host-side mirror of the reference's patch strategy
(enlightning.C) used to drive it.
"""
from .constants import VARIANTS, default_params  # noqa: F401

__all__ = ["VARIANTS", "default_params"]
