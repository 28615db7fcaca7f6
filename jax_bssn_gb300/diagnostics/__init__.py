"""Wave and constraint diagnostics and output staging on GB300 (mirrors JAX_BSSN/diagnostics)."""

from .openpmd import stage_output_fields, strip_ghost_cells, tiled_output_fields
from .waves import composite_wave_diagnostics, diagnostic_fields, h_plus

__all__ = ["composite_wave_diagnostics", "diagnostic_fields", "h_plus", "stage_output_fields",
           "strip_ghost_cells", "tiled_output_fields"]
