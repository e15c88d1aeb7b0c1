"""GB300-native SGH (staggered-grid hydrodynamics) Lagrangian cycle for 3D hex
meshes: a drop-in for the sgh_solve hot path of Fierro's Explicit-Lagrange-Kokkos
SGH solver.  The compute path is libfierro_sgh.so (hand-written sm_103a CUDA
behind the C ABI in include/fierro_sgh.h); ``fierro_gb300.sgh`` is its Python
mirror and loads the library on import (there is no CPU fallback).
"""
from . import mesh, problems  # noqa: F401

__all__ = ["mesh", "problems", "sgh"]
