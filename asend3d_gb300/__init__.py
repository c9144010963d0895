"""GB300-native (sm_103a) linear-elastic static / Newmark / adjoint solve path.

Drop-in for the solve core of MSDOToolz/ASenD3D: the C ABI in
include/asend_gpu.h (libasend_gpu.so, built in-tree by asend3d_gb300.build)
plus a Python host mirror of the reference's model / load / design-variable /
objective interface (asend3d_gb300.solver).
"""
from .mesh import BlockMesh, block_hex8, block_tet4, lognormal_modulus  # noqa: F401
from .solver import AsendError, GpuSolver, Problem  # noqa: F401

__all__ = ["BlockMesh", "block_hex8", "block_tet4", "lognormal_modulus", "AsendError", "GpuSolver", "Problem"]
