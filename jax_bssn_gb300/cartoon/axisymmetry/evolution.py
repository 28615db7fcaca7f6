"""Stage-wise z-axis axisymmetric Cartoon evolution (mirrors JAX_BSSN/cartoon/axisymmetry/evolution.py).

Both entry points run entirely in ``libbssn_gb300.so``: reconstruction onto
the nine-plane support, the Cartesian RHS on the centre plane only (every
stencil reaches at most four samples in y, so the centre plane never sees the
support's periodic wrap and equals the reference's full-support RHS there),
collection into compact storage, and the RK4 stage epilogues with the
algebraic projection and parity-ghost refill of ``_prepare_stage``.
"""

from __future__ import annotations

from ...bssn.variables import BSSNParameters, BSSNVariables
from .. import _calls


def compute_axisymmetric_rhs(vars: BSSNVariables, params: BSSNParameters) -> BSSNVariables:
    """Compact RHS with parity ghosts (evolution.py:18-26)."""
    return _calls.rhs(vars, params, axi=True)


def axisymmetric_rk4_step(vars: BSSNVariables, params: BSSNParameters) -> BSSNVariables:
    """One classical RK4 step with per-stage projection and ghost refill (evolution.py:40-65)."""
    return _calls.rk4(vars, params, axi=True)


def axisymmetric_rk4_steps(vars: BSSNVariables, params: BSSNParameters, steps: int) -> BSSNVariables:
    """``steps`` repetitions of ``axisymmetric_rk4_step`` in one device call."""
    return _calls.rk4(vars, params, axi=True, steps=steps)


class AxisymmetricEvolution(_calls.CartoonEvolution):
    """Resident compact axisymmetric state: ``step(n)`` without layout conversion."""

    def __init__(self, vars: BSSNVariables, params: BSSNParameters, precision: str | None = None):
        super().__init__(vars, params, axisymmetric=True, precision=precision)


__all__ = ["AxisymmetricEvolution", "axisymmetric_rk4_step", "axisymmetric_rk4_steps", "compute_axisymmetric_rhs"]
