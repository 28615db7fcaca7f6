"""Wave and constraint diagnostics on GB300 (mirrors JAX_BSSN/diagnostics)."""

from .waves import composite_wave_diagnostics, diagnostic_fields, h_plus

__all__ = ["composite_wave_diagnostics", "diagnostic_fields", "h_plus"]
