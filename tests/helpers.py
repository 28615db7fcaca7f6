"""Shared helpers: golden fixtures, parameter conversion, per-field errors."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
LEAVES = ("conformal_metric", "conformal_factor", "traceless_K", "trace_K",
          "conformal_connection", "lapse", "shift")


def load_golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as data:
        return {k: data[k] for k in data.files}


def golden_state(data: dict, prefix: str, cls):
    return cls(*(data[f"{prefix}.{leaf}"] for leaf in LEAVES))


def golden_params(data: dict, cls):
    raw = json.loads(str(data["params"]))
    for key in ("owned_shape", "owned_faces", "reduced_axes"):
        if isinstance(raw.get(key), list):
            raw[key] = tuple(raw[key])
    return cls(**raw)


def field_errors(a, b, floor: float = 1e-300) -> dict:
    """max|a-b| / max(max|b|, floor) per leaf (norm-relative)."""
    out = {}
    for leaf, x, y in zip(LEAVES, a, b):
        x = np.asarray(x.detach().cpu().numpy() if hasattr(x, "detach") else x, dtype=np.float64)
        y = np.asarray(y.detach().cpu().numpy() if hasattr(y, "detach") else y, dtype=np.float64)
        scale = max(float(np.max(np.abs(y))), floor)
        out[leaf] = float(np.max(np.abs(x - y))) / scale
    return out


def worst(errors: dict) -> float:
    return max(errors.values())


RHS_CASES = ("gauge_wave", "generic_kappa", "sommerfeld", "mad_mixed", "mad_periodic_zero_shift",
             "boosted_weak_wave")


def assert_norms_match(got: dict, ref: dict, rel: float = 1e-9) -> None:
    """Constraint norms against the reference's.  det(gt)-1 and tr(At) vanish
    for projected data up to roundoff of O(1) products, so their norms are
    compared absolutely at that O(1) scale; the others relatively."""
    for key, value in ref.items():
        if key.startswith(("det_gamma", "trace_A")):
            assert abs(got[key] - value) < 1e-14, (key, got[key], value)
        else:
            assert abs(got[key] - value) <= rel * abs(value) + 1e-18, (key, got[key], value)
