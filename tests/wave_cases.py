"""Shared inputs of the wave-diagnostics tests: the golden archive's tree and
the two known-answer trees of the reference's own suite
(tests/FMR/test_wave_demo.py:33-92), with their closed-form answers."""

from __future__ import annotations

import json
import math

import numpy as np

from .helpers import load_golden


def golden_tree(spec_cls, hierarchy_cls):
    data = load_golden("waves")
    specs = tuple(spec_cls(tuple(lo), tuple(hi), parent=parent)
                  for lo, hi, parent in json.loads(str(data["tree.hierarchy"])))
    hierarchy = hierarchy_cls(specs)
    levels, coords = [], []
    for i in range(len(specs) + 1):
        levels.append({"h_plus": data[f"tree.{i}.h_plus"], "hamiltonian_constraint": data[f"tree.{i}.hamiltonian"],
                       "momentum_constraint": tuple(data[f"tree.{i}.momentum"])})
        coords.append(data[f"tree.{i}.x"])
    time, amplitude, wavelength = (float(v) for v in data["tree.scalars"])
    keys = json.loads(str(data["tree.keys"]))
    expect = {"active": dict(zip(keys, data["tree.active"])), "guarded": dict(zip(keys, data["tree.guarded"]))}
    return hierarchy, levels, coords, (time, amplitude, wavelength), expect


def padded(hierarchy, levels, coords):
    out, xs = [levels[0]], [coords[0]]
    for lv, x, spec in zip(levels[1:], coords[1:], hierarchy.patches):
        g = spec.ghost_width
        pad = lambda a: np.pad(np.asarray(a), g, constant_values=999.0)  # noqa: E731
        out.append({"h_plus": pad(lv["h_plus"]), "hamiltonian_constraint": pad(lv["hamiltonian_constraint"]),
                    "momentum_constraint": tuple(pad(m) for m in lv["momentum_constraint"])})
        xs.append(pad(x))
    return out, xs


def vertex_count_tree(spec_cls, hierarchy_cls):
    """One child over root vertices [1,3]x[1,3]x[1,2]; 999 on the covered box."""
    hierarchy = hierarchy_cls((spec_cls((1, 1, 1), (3, 3, 2)),))
    root, child = np.ones((6, 5, 4)), np.ones((5, 5, 3))
    error = 2 * root
    error[1:4, 1:4, 1:3] = 999.0
    fields = ({"h_plus": error, "hamiltonian_constraint": 5 * root, "momentum_constraint": (root, 2 * root, 2 * root)},
              {"h_plus": 3 * child, "hamiltonian_constraint": 7 * child,
               "momentum_constraint": (2 * child, 3 * child, 6 * child)})
    coords = (0 * root, 0 * child)
    nr, nc = 120 - 18, 75
    n = nr + nc
    answer = {"composite_rms": math.sqrt((nr * 4 + nc * 9) / n), "composite_max": 3.0,
              "composite_hamiltonian_l2": math.sqrt((nr * 25 + nc * 49) / n),
              "composite_momentum_l2": math.sqrt((nr * 9 + nc * 49) / n)}
    return hierarchy, fields, coords, answer


def branching_tree(spec_cls, hierarchy_cls):
    """Two siblings under the root and a grandchild under the first sibling;
    coverage is per parent."""
    hierarchy = hierarchy_cls((spec_cls((1, 1, 1), (3, 3, 3), parent=0), spec_cls((4, 1, 1), (6, 3, 3), parent=0),
                               spec_cls((1, 1, 1), (3, 3, 3), parent=1)))
    shapes = ((8,) * 3,) + ((5,) * 3,) * 3
    covered = ((slice(1, 4),) * 3, (slice(4, 7),) + (slice(1, 4),) * 2)
    values = (1.0, 2.0, 3.0, 4.0)
    fields = []
    for patch, (shape, value) in enumerate(zip(shapes, values)):
        wave, hamiltonian = np.full(shape, value), np.full(shape, value + 4.0)
        boxes = covered if patch == 0 else (covered[0],) if patch == 1 else ()
        for box in boxes:
            wave[box] = 999.0
            hamiltonian[box] = 999.0
        fields.append({"h_plus": wave, "hamiltonian_constraint": hamiltonian, "momentum_constraint": (wave,) * 3})
    coords = tuple(np.zeros(shape) for shape in shapes)
    counts = (8 ** 3 - 2 * 3 ** 3, 5 ** 3 - 3 ** 3, 5 ** 3, 5 ** 3)
    total = sum(counts)
    answer = {"composite_rms": math.sqrt(sum(n * v ** 2 for n, v in zip(counts, values)) / total),
              "composite_max": 4.0,
              "composite_hamiltonian_l2": math.sqrt(sum(n * (v + 4) ** 2 for n, v in zip(counts, values)) / total),
              "composite_momentum_l2": math.sqrt(3 * sum(n * v ** 2 for n, v in zip(counts, values)) / total)}
    return hierarchy, tuple(fields), coords, answer


def assert_close(got: dict, expect: dict, rel: float) -> None:
    for key, value in expect.items():
        assert abs(got[key] - value) <= rel * abs(value) + 1e-300, (key, got[key], value)
