"""Vertex-centred 2:1 patch geometry (mirrors JAX_BSSN/fmr/refinement.py:15-85)."""

from __future__ import annotations

from typing import NamedTuple


class FMRPatchSpec(NamedTuple):
    """Inclusive parent-active-index bounds of one child patch."""
    coarse_lo: tuple
    coarse_hi: tuple
    refinement_ratio: int = 2
    ghost_width: int = 4
    parent: int | None = None


class FMRHierarchySpec(NamedTuple):
    """Parent-before-child patches and the hierarchy-wide MAD choice."""
    patches: tuple
    use_mad: bool = True


def hierarchy_parents(hierarchy) -> tuple:
    """Flat parent index of every patch; the root is -1 (refinement.py:32-49)."""
    parents = [-1]
    for child, spec in enumerate(hierarchy.patches, start=1):
        parent = child - 1 if spec.parent is None else spec.parent
        if not isinstance(parent, int) or not 0 <= parent < child:
            raise ValueError("FMR patches must follow their parent in the hierarchy")
        parents.append(int(parent))
    for child, spec in enumerate(hierarchy.patches, start=1):
        for other in range(1, child):
            sibling = hierarchy.patches[other - 1]
            if parents[child] == parents[other] and all(
                    max(a, b) <= min(c, d) for a, b, c, d in
                    zip(spec.coarse_lo, sibling.coarse_lo, spec.coarse_hi, sibling.coarse_hi)):
                raise ValueError("sibling FMR patches must not share owned vertices")
    return tuple(parents)


def hierarchy_depths(hierarchy) -> tuple:
    depths = [0]
    for parent in hierarchy_parents(hierarchy)[1:]:
        depths.append(depths[parent] + 1)
    return tuple(depths)


def _validate_spec(spec) -> None:
    if len(spec.coarse_lo) != 3 or len(spec.coarse_hi) != 3:
        raise ValueError("FMR patch bounds must be three-dimensional")
    if spec.refinement_ratio != 2:
        raise ValueError("FMR refinement ratio must be 2:1")
    if spec.ghost_width != 4:
        raise ValueError("the BSSN FMR configuration requires four guard cells")
    if any(h < l for l, h in zip(spec.coarse_lo, spec.coarse_hi)):
        raise ValueError("coarse_hi must not precede coarse_lo")


def fine_active_shape(spec) -> tuple:
    _validate_spec(spec)
    return tuple(2 * (h - l) + 1 for l, h in zip(spec.coarse_lo, spec.coarse_hi))


def fine_active_slice(spec) -> tuple:
    g = spec.ghost_width
    return tuple(slice(g, g + n) for n in fine_active_shape(spec))


def fine_active_view(array, spec):
    return array[(...,) + fine_active_slice(spec)]
