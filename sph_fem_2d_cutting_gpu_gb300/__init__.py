"""GB300-native (sm_103a) SPH workpiece hot path of the hybrid SPH-FEM 2D
cutting solver: cell list, neighbour sums, Johnson-Cook plasticity,
leap-frog update and FEM-tool contact / heat coupling, behind the C ABI of
include/sphfem.h.  ``sph_fem_2d_cutting_gpu_gb300.build.build()`` compiles the
CUDA library in-tree; ``solver.Solver`` drives it."""
