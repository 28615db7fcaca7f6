"""BSSN state contract (mirrors JAX_BSSN.bssn)."""

from .variables import BSSNParameters, BSSNVariables, get_boundary_codes

__all__ = ["BSSNParameters", "BSSNVariables", "get_boundary_codes"]
