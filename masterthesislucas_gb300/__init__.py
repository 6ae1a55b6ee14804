"""GB300-native 2D tree code (symmetric Morton FMM, direct sums, t-SNE step).

The compute path is libtreecode.so (hand-written sm_103a CUDA behind the C
ABI in include/treecode.h); this package is its host-side mirror of the
reference's solver and t-SNE interfaces.
"""
from .solver import (NBodySolverFMM_MORTON, NBodySolverFMM_SYM_MORTON, NBodySolverPM, Points, direct,  # noqa: F401
                     get_depth, node_count, particle_mesh)

__all__ = ["NBodySolverFMM_MORTON", "NBodySolverFMM_SYM_MORTON", "NBodySolverPM", "Points", "direct", "get_depth",
           "node_count", "particle_mesh"]
