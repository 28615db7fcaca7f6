"""Spherical Cartoon on GB300 (mirrors JAX_BSSN.cartoon.spherical_symmetry)."""

from .diagnostics import (cartoon_axis_output_fields, compute_cartoon_constraint_norms, compute_cartoon_constraints,
                          compute_spherical_symmetry_norms)
from .evolution import SphericalEvolution, cartoon_rk4_step, cartoon_rk4_steps, compute_cartoon_rhs
from .reconstruction import (CARTOON_CENTER, CARTOON_GHOST_CELLS, CARTOON_OUTER_BUFFER_CELLS, CARTOON_SUPPORT_SIZE,
                             RADIAL_VECTOR_PARITY, cartoon_centerline, cartoon_positive_radius, compact_cartoon_state,
                             enforce_spherical_symmetry, expand_cartoon_axis, expand_cartoon_scalar,
                             expand_cartoon_vector, project_cartoon_rhs, project_cartoon_scalar,
                             project_cartoon_vector, radial_interpolate, reconstruct_cartoon_support,
                             transformation_matrix, validate_cartoon_grid)

__all__ = [
    "CARTOON_CENTER", "CARTOON_GHOST_CELLS", "CARTOON_OUTER_BUFFER_CELLS", "CARTOON_SUPPORT_SIZE",
    "RADIAL_VECTOR_PARITY", "SphericalEvolution", "cartoon_axis_output_fields", "cartoon_centerline",
    "cartoon_positive_radius", "cartoon_rk4_step", "cartoon_rk4_steps", "compact_cartoon_state",
    "compute_cartoon_constraint_norms", "compute_cartoon_constraints", "compute_spherical_symmetry_norms",
    "compute_cartoon_rhs", "enforce_spherical_symmetry", "expand_cartoon_axis", "expand_cartoon_scalar",
    "expand_cartoon_vector", "project_cartoon_rhs", "project_cartoon_scalar", "project_cartoon_vector",
    "radial_interpolate", "reconstruct_cartoon_support", "transformation_matrix", "validate_cartoon_grid",
]
