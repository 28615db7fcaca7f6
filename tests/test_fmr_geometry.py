"""Host-side FMR patch geometry: the reference suite's known answers
(JAX_BSSN tests/FMR/test_fmr_geometry.py:21-46), restated on the package."""

import numpy as np
import pytest

from jax_bssn_gb300.fmr.refinement import (FMRHierarchySpec, FMRPatchSpec, fine_active_shape,
                                           fine_active_slice, fine_active_view, hierarchy_depths,
                                           hierarchy_parents)


def test_inclusive_bounds_give_odd_extents_and_guarded_views():
    spec = FMRPatchSpec((4, 4, 4), (9, 9, 9))
    assert fine_active_shape(spec) == (11, 11, 11)
    assert fine_active_slice(spec) == (slice(4, 15),) * 3
    padded = np.arange(19.0 ** 3).reshape((19,) * 3)
    view = fine_active_view(padded, spec)
    assert view.shape == (11, 11, 11)
    assert np.array_equal(view, padded[4:15, 4:15, 4:15])
    tensor = np.broadcast_to(padded, (3, 3) + padded.shape)
    assert fine_active_view(tensor, spec).shape == (3, 3, 11, 11, 11)
    assert fine_active_shape(FMRPatchSpec((32, 20, 0), (64, 44, 0))) == (65, 49, 1)


def test_explicit_parents_depths_and_sibling_ownership():
    left = FMRPatchSpec((2, 2, 2), (6, 6, 6), parent=0)
    right = FMRPatchSpec((7, 2, 2), (11, 6, 6), parent=0)
    grandchild = FMRPatchSpec((2, 2, 2), (4, 4, 4), parent=1)
    hierarchy = FMRHierarchySpec((left, grandchild, right))
    assert hierarchy_parents(hierarchy) == (-1, 0, 1, 0)
    assert hierarchy_depths(hierarchy) == (0, 1, 2, 1)
    # bounds are inclusive: touching at x = 6 shares a vertex
    with pytest.raises(ValueError, match="share owned vertices"):
        hierarchy_parents(FMRHierarchySpec((left, right._replace(coarse_lo=(6, 2, 2)))))
    with pytest.raises(ValueError, match="follow their parent"):
        hierarchy_parents(FMRHierarchySpec((left._replace(parent=1),)))
    # omitted parents chain each patch to the one before it
    chain = FMRHierarchySpec((FMRPatchSpec((32,) * 3, (64,) * 3), FMRPatchSpec((20,) * 3, (44,) * 3)))
    assert hierarchy_parents(chain) == (-1, 0, 1)
    assert hierarchy_depths(chain) == (0, 1, 2)
    # numpy integers are accepted as parent indices
    assert hierarchy_parents(FMRHierarchySpec((left._replace(parent=np.int64(0)),))) == (-1, 0)
    # siblings of different parents may overlap in index space
    cousin = grandchild._replace(parent=3)
    assert hierarchy_parents(FMRHierarchySpec((left, grandchild, right, cousin))) == (-1, 0, 1, 0, 3)


@pytest.mark.parametrize("spec, message", [
    (FMRPatchSpec((1, 1), (2, 2)), "three-dimensional"),
    (FMRPatchSpec((1, 1, 1), (2, 2, 2), refinement_ratio=4), "2:1"),
    (FMRPatchSpec((1, 1, 1), (2, 2, 2), ghost_width=3), "four guard cells"),
    (FMRPatchSpec((3, 1, 1), (2, 2, 2)), "must not precede"),
])
def test_invalid_specs_raise_the_reference_messages(spec, message):
    with pytest.raises(ValueError, match=message):
        fine_active_shape(spec)
