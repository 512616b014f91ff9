"""GB300-native matrix-free voxel-elasticity MGPCG solver (SGLDBench solve path).

The compute path is the CUDA library ``libsgld_gb300.so`` (C ABI in
``include/sgld_gpu.h``); ``VoxelSolver`` is the Python host interface over it.
Importing the package does not load the library; constructing a solver does,
and fails loudly when it is not built.
"""
from .solver import LoadCases, VoxelSolver, pad_voxels, reference_num_levels, simp_modulus  # noqa: F401

__all__ = ["LoadCases", "VoxelSolver", "pad_voxels", "reference_num_levels", "simp_modulus"]
