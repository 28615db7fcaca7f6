"""Puncture initial data and the apparent-horizon finder on the GPU (mirrors JAX_BSSN/utilities)."""

from .bowen_york_solver import (  # noqa: F401
    PunctureSolve,
    axisymmetric_cell_centered_grid,
    axisymmetric_hamiltonian_residual,
    axisymmetric_laplacian,
    axisymmetric_linearized_hamiltonian_operator,
    bowen_york_extrinsic_curvature,
    brill_lindquist_conformal_factor,
    cell_centered_grid,
    contract_conformal_curvature,
    hamiltonian_residual,
    hamiltonian_source,
    laplacian,
    linearized_hamiltonian_operator,
    linearized_hamiltonian_source,
    puncture_solve,
    solve_axisymmetric_conformal_factor,
    solve_conformal_factor,
)
from .apparent_horizon import (  # noqa: F401
    ExpansionResidual,
    angular_derivatives,
    angular_grid,
    build_geometry,
    dense_jacobian,
    find_apparent_horizon,
    interpolate_angular,
    surface,
    theta_ghosts,
)
