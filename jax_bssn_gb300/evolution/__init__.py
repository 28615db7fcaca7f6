"""Time integration on GB300 (mirrors JAX_BSSN.evolution)."""

from .time_evolve import (compute_bssn_rhs, compute_bssn_rhs_with_matter,
                          enforce_algebraic_constraints, rk4_step, rk4_steps)
from .resident import BatchEvolution, NonFiniteStateError, PatchEvolution

__all__ = ["compute_bssn_rhs", "compute_bssn_rhs_with_matter", "enforce_algebraic_constraints",
           "rk4_step", "rk4_steps", "PatchEvolution", "BatchEvolution", "NonFiniteStateError"]
