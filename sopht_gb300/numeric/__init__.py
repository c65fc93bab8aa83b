"""Eulerian grid and immersed-boundary operators (sopht.numeric counterparts)."""

from . import eulerian_grid_ops, immersed_boundary_ops
from .eulerian_grid_ops import (
    UnboundedPoissonSolver2D,
    UnboundedPoissonSolver3D,
    UnboundedPoissonSolverPYFFTW2D,
    UnboundedPoissonSolverPYFFTW3D,
)
from .immersed_boundary_ops import VirtualBoundaryForcing

__all__ = [
    "UnboundedPoissonSolver2D",
    "UnboundedPoissonSolver3D",
    "UnboundedPoissonSolverPYFFTW2D",
    "UnboundedPoissonSolverPYFFTW3D",
    "VirtualBoundaryForcing",
    "eulerian_grid_ops",
    "immersed_boundary_ops",
]
