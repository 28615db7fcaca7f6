"""Vertex-centred 2:1 patch geometry of the FMR hierarchy.

Interface of JAX_BSSN/fmr/refinement.py:15-85: the two spec tuples (same
fields and defaults), the parent/depth queries and the fine-patch extent
helpers, with the reference's ValueError messages (its tests match on them).

A child patch owns both of its inclusive parent bounds, so along each axis it
has 2 * (hi - lo) + 1 active vertices, stored after four guard samples.
"""

from __future__ import annotations

import numbers
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


def _parent_index(spec: FMRPatchSpec, position: int) -> int:
    """Parent of the patch at flat ``position`` (>= 1); omitted means the
    patch just before it, which keeps the older single-chain hierarchies."""
    parent = position - 1 if spec.parent is None else spec.parent
    if isinstance(parent, numbers.Integral) and 0 <= parent < position:
        return int(parent)
    raise ValueError("FMR patches must follow their parent in the hierarchy")


def _boxes_meet(a: FMRPatchSpec, b: FMRPatchSpec) -> bool:
    """True when the closed boxes [lo, hi] of two patches share a vertex:
    their index intervals intersect on every axis."""
    return all(not (a_hi < b_lo or b_hi < a_lo)
               for a_lo, a_hi, b_lo, b_hi in zip(a.coarse_lo, a.coarse_hi, b.coarse_lo, b.coarse_hi))


def _tree(hierarchy) -> tuple[tuple, tuple]:
    """Parents and depths of every flat patch (root first: parent -1, depth 0).

    All parent links are checked before any sibling overlap, so a hierarchy
    with both faults reports the broken link, as the reference does.
    """
    specs = tuple(hierarchy.patches)
    parents = (-1,) + tuple(_parent_index(spec, pos) for pos, spec in enumerate(specs, start=1))
    children_of: dict[int, list[FMRPatchSpec]] = {}
    for pos, spec in enumerate(specs, start=1):
        family = children_of.setdefault(parents[pos], [])
        if any(_boxes_meet(spec, earlier) for earlier in family):
            raise ValueError("sibling FMR patches must not share owned vertices")
        family.append(spec)
    depths = [0]
    for parent in parents[1:]:
        depths.append(depths[parent] + 1)
    return parents, tuple(depths)


def hierarchy_parents(hierarchy) -> tuple:
    """Flat parent index of every patch; the root is -1."""
    return _tree(hierarchy)[0]


def hierarchy_depths(hierarchy) -> tuple:
    """Refinement level of every flat patch; the root is 0."""
    return _tree(hierarchy)[1]


def _check_spec(spec: FMRPatchSpec) -> None:
    lo, hi = tuple(spec.coarse_lo), tuple(spec.coarse_hi)
    if (len(lo), len(hi)) != (3, 3):
        raise ValueError("FMR patch bounds must be three-dimensional")
    if spec.refinement_ratio != 2:
        raise ValueError("FMR refinement ratio must be 2:1")
    if spec.ghost_width != 4:
        raise ValueError("the BSSN FMR configuration requires four guard cells")
    if min(h - l for l, h in zip(lo, hi)) < 0:
        raise ValueError("coarse_hi must not precede coarse_lo")


def fine_active_shape(spec: FMRPatchSpec) -> tuple:
    """Active vertices of the child along each axis: both parent bounds are
    owned, and every parent interval holds one new midpoint."""
    _check_spec(spec)
    return tuple(1 + spec.refinement_ratio * (h - l) for l, h in zip(spec.coarse_lo, spec.coarse_hi))


def fine_active_slice(spec: FMRPatchSpec) -> tuple:
    """Slices of the active vertices inside the child's guarded array."""
    start = spec.ghost_width
    return tuple(slice(start, start + n) for n in fine_active_shape(spec))


def fine_active_view(array, spec: FMRPatchSpec):
    """The active vertices of a guarded child array (leading axes kept)."""
    return array[(Ellipsis, *fine_active_slice(spec))]
