"""Stage-wise spherical Cartoon evolution (mirrors JAX_BSSN/cartoon/spherical_symmetry/evolution.py).

Reconstruction onto the 9 x 9 support, the Cartesian RHS on the centre line
only (stencils reach four samples in y and z, so the centre line never sees
the support's periodic wrap), and the RK4 stage epilogues -- symmetric
subspace first, then the algebraic projection, then the parity ghosts -- all
run in ``libbssn_gb300.so``.
"""

from __future__ import annotations

from ...bssn.variables import BSSNParameters, BSSNVariables
from .. import _calls


def compute_cartoon_rhs(vars: BSSNVariables, params: BSSNParameters) -> BSSNVariables:
    """Compact RHS with parity ghosts (evolution.py:17-25)."""
    return _calls.rhs(vars, params, axi=False)


def cartoon_rk4_step(vars: BSSNVariables, params: BSSNParameters) -> BSSNVariables:
    """One classical RK4 step with the spherical stage preparation (evolution.py:44-72)."""
    return _calls.rk4(vars, params, axi=False)


def cartoon_rk4_steps(vars: BSSNVariables, params: BSSNParameters, steps: int) -> BSSNVariables:
    """``steps`` repetitions of ``cartoon_rk4_step`` in one device call."""
    return _calls.rk4(vars, params, axi=False, steps=steps)


class SphericalEvolution(_calls.CartoonEvolution):
    """Resident compact spherical state: ``step(n)`` without layout conversion."""

    def __init__(self, vars: BSSNVariables, params: BSSNParameters, precision: str | None = None):
        super().__init__(vars, params, axisymmetric=False, precision=precision)


__all__ = ["SphericalEvolution", "cartoon_rk4_step", "cartoon_rk4_steps", "compute_cartoon_rhs"]
