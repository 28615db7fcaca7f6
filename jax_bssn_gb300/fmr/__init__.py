"""Fixed mesh refinement on GB300 (mirrors JAX_BSSN.fmr)."""

from .refinement import (FMRHierarchySpec, FMRPatchSpec, fine_active_shape, fine_active_slice,
                         fine_active_view, hierarchy_depths, hierarchy_parents)
from .tiled import (FMREvolution, TileLayout, evolution_parameters, fmr_constraint_norms, fmr_rk4_step,
                    fmr_rk4_steps, fmr_stage, initialize_tiled_fmr, patch_layout, prepare_fmr_states,
                    validate_hierarchy)
from .transfer import fill_tiled_fine_ghosts, restrict_tiled_to_coarse

__all__ = ["FMRHierarchySpec", "FMRPatchSpec", "fine_active_shape", "fine_active_slice", "fine_active_view",
           "hierarchy_depths", "hierarchy_parents", "FMREvolution", "TileLayout", "evolution_parameters",
           "fmr_constraint_norms", "fmr_rk4_step", "fmr_rk4_steps", "fmr_stage", "initialize_tiled_fmr",
           "patch_layout", "prepare_fmr_states", "validate_hierarchy", "fill_tiled_fine_ghosts",
           "restrict_tiled_to_coarse"]
