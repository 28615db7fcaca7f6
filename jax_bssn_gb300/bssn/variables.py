"""BSSN state and parameter containers, field-for-field the reference contract.

JAX_BSSN/bssn/variables.py:8-59: seven leaves in a fixed numerical order, and
a NamedTuple of scalar parameters including the tile description used by the
tiled and FMR paths.  Leaves may be CUDA tensors or host arrays.
"""

from typing import NamedTuple, Tuple


class BSSNVariables(NamedTuple):
    """Evolved fields: gamma_tilde (3,3,...), W, A_tilde (3,3,...), K,
    Gamma_tilde (3,...), alpha, beta (3,...)."""
    conformal_metric: object
    conformal_factor: object
    traceless_K: object
    trace_K: object
    conformal_connection: object
    lapse: object
    shift: object


class BSSNParameters(NamedTuple):
    eta: float = 2.0
    kappa: float = 0.0
    nu: float = 0.002
    g: float = 0.75
    dx: float = 0.1
    dt: float = 0.001
    zero_shift: int = 0
    gauge: int = 0
    xl_bc: int = 0
    xr_bc: int = 0
    yl_bc: int = 0
    yr_bc: int = 0
    zl_bc: int = 0
    zr_bc: int = 0
    x_min: float = 0.0
    y_min: float = 0.0
    z_min: float = 0.0
    mad_q: float = 1.0
    guard_cells: int = 0
    owned_shape: tuple | None = None
    owned_faces: tuple = (True, True, True, True, True, True)
    reduced_axes: tuple | None = None


def get_boundary_codes(params: BSSNParameters, spatial_direction: int) -> Tuple[int, int]:
    """Left and right face codes of one direction (JAX_BSSN/bssn/variables.py:49-59)."""
    if spatial_direction == 0:
        return params.xl_bc, params.xr_bc
    if spatial_direction == 1:
        return params.yl_bc, params.yr_bc
    return params.zl_bc, params.zr_bc
