"""Wave diagnostics restated in NumPy (test infrastructure).

Follows uwplasma/JAX_BSSN/diagnostics/waves.py:
  h_plus                       :11-20   0.5 (gt_yy / W**2 - gt_zz / W**2)
  diagnostic_fields            :23-39   h_plus, gauge fields, H and M_i
  composite_wave_diagnostics   :43-91   point-count norms over the vertices of
                                        each level that no child of that level
                                        covers
Only the tests and the bench's CPU legs import this module.
"""

from __future__ import annotations

import math

import numpy as np

from . import bssn as ob
from .fmr import fine_active_shape, parents_of


def h_plus(v):
    W = np.asarray(v.conformal_factor)
    g = np.asarray(v.conformal_metric)
    return 0.5 * (g[1, 1] / W ** 2 - g[2, 2] / W ** 2)


def diagnostic_fields(v, p):
    H, M, _, _, _ = ob.constraints(v, p)
    return {
        "h_plus": h_plus(v),
        "lapse": np.asarray(v.lapse),
        "shift": tuple(np.asarray(v.shift)[i] for i in range(3)),
        "K": np.asarray(v.trace_K),
        "W": np.asarray(v.conformal_factor),
        "hamiltonian_constraint": H,
        "momentum_constraint": tuple(M[i] for i in range(3)),
    }


def _active(a, spec):
    g = spec.ghost_width
    return np.asarray(a)[(...,) + tuple(slice(g, g + m) for m in fine_active_shape(spec))]


def composite_wave_diagnostics(level_fields, level_coordinates, hierarchy, time, amplitude, wavelength, *,
                               active_fields=False):
    parents = parents_of(hierarchy)
    error_sum = hamiltonian_sum = momentum_sum = 0.0
    maximum = 0.0
    point_count = 0
    for level, (fields, coordinates) in enumerate(zip(level_fields, level_coordinates)):
        h = np.asarray(fields["h_plus"])
        H = np.asarray(fields["hamiltonian_constraint"])
        M = [np.asarray(m) for m in fields["momentum_constraint"]]
        x = np.asarray(coordinates)
        if level and not active_fields:
            spec = hierarchy.patches[level - 1]
            h, H, x = _active(h, spec), _active(H, spec), _active(x, spec)
            M = [_active(m, spec) for m in M]
        mask = np.ones(h.shape, dtype=bool)
        for child_index, parent in enumerate(parents[1:], start=1):
            if parent == level:
                child = hierarchy.patches[child_index - 1]
                mask[tuple(slice(lo, hi + 1) for lo, hi in zip(child.coarse_lo, child.coarse_hi))] = False
        exact = amplitude * np.sin(2.0 * np.pi * (x - time) / wavelength)
        error = h - exact
        error_sum += float(np.sum(np.where(mask, error ** 2, 0.0)))
        hamiltonian_sum += float(np.sum(np.where(mask, H ** 2, 0.0)))
        momentum_sum += float(np.sum(np.where(mask, sum(m ** 2 for m in M), 0.0)))
        maximum = max(maximum, float(np.max(np.where(mask, np.abs(error), 0.0))))
        point_count += int(np.sum(mask))
    rms = math.sqrt(error_sum / point_count)
    return {
        "composite_rms": rms,
        "composite_max": maximum,
        "composite_hamiltonian_l2": math.sqrt(hamiltonian_sum / point_count),
        "composite_momentum_l2": math.sqrt(momentum_sum / point_count),
        "coarse_rms": rms,
        "fine_rms": rms,
    }
