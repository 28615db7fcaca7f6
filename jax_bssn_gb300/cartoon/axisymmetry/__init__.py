"""z-axis axisymmetric Cartoon on GB300 (mirrors JAX_BSSN.cartoon.axisymmetry)."""

from .diagnostics import (axisymmetric_plane_output_fields, compute_axisymmetric_constraint_norms,
                          compute_axisymmetric_constraints)
from .evolution import AxisymmetricEvolution, axisymmetric_rk4_step, axisymmetric_rk4_steps, compute_axisymmetric_rhs
from .reconstruction import (compact_axisymmetric_state, expand_axisymmetric_plane, expand_axisymmetric_scalar,
                             expand_axisymmetric_vector, fill_axisymmetric_ghosts, project_axisymmetric_rhs,
                             project_axisymmetric_scalar, project_axisymmetric_vector, radial_interpolate,
                             reconstruct_axisymmetric_support, transformation_matrix, validate_axisymmetric_grid)

__all__ = [
    "AxisymmetricEvolution", "axisymmetric_plane_output_fields", "axisymmetric_rk4_step", "axisymmetric_rk4_steps",
    "compact_axisymmetric_state", "compute_axisymmetric_constraint_norms", "compute_axisymmetric_constraints",
    "compute_axisymmetric_rhs", "expand_axisymmetric_plane", "expand_axisymmetric_scalar",
    "expand_axisymmetric_vector", "fill_axisymmetric_ghosts", "project_axisymmetric_rhs",
    "project_axisymmetric_scalar", "project_axisymmetric_vector", "radial_interpolate",
    "reconstruct_axisymmetric_support", "transformation_matrix", "validate_axisymmetric_grid",
]
