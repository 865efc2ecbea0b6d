"""GB300-native (sm_103a) SPH workpiece hot path of the hybrid SPH-FEM 2D
cutting solver: cell list, neighbour sums, Johnson-Cook plasticity,
leap-frog update and FEM-tool contact / heat coupling, behind the C ABI of
include/sphfem.h.  ``build()`` compiles the CUDA library in-tree."""
from .build import build  # noqa: F401

__all__ = ["build"]
