"""GB300 (sm_103a) implementation of PANSFEM2's SIMP topology-optimisation loop.

The compute path is the CUDA library built from pansfem2_gb300/csrc (C ABI in
include/pansfem2_gpu.h).  This package is a thin Python host over that ABI;
the C++ host mirror of the reference's template API is include/pansfem2_gb300.hpp.
"""
from . import problems  # noqa: F401
from ._lib import PsfError, SOLVERS, kernel_launches, load  # noqa: F401
from .api import DeviceMMA, Problem  # noqa: F401
