"""Load FMR golden archives into oracle-shaped inputs."""

from __future__ import annotations

import json

import numpy as np

from oracle import fmr as ofmr
from oracle.state import BSSNParameters, BSSNVariables

from .helpers import LEAVES, load_golden

G = ofmr.GUARD


def hierarchy_of(data):
    h = json.loads(str(data["hierarchy"]))
    patches = tuple(ofmr.FMRPatchSpec(tuple(lo), tuple(hi), parent=parent) for lo, hi, parent in h["patches"])
    return ofmr.FMRHierarchySpec(patches, use_mad=h["use_mad"])


def root_params_of(data, cls=BSSNParameters):
    raw = json.loads(str(data["root_params"]))
    for key in ("owned_shape", "owned_faces", "reduced_axes"):
        if isinstance(raw.get(key), list):
            raw[key] = tuple(raw[key])
    return cls(**raw)


def owned_states(data, prefix, count):
    return tuple(BSSNVariables(*(data[f"{prefix}.{p}.{leaf}"] for leaf in LEAVES)) for p in range(count))


def padded_from_owned(owned_state, n):
    leaves = []
    for leaf in owned_state:
        a = np.asarray(leaf)
        full = np.zeros(a.shape[:-3] + tuple(m + 2 * G for m in n))
        full[(Ellipsis,) + tuple(slice(G, G + m) for m in n)] = a
        leaves.append(full)
    return BSSNVariables(*leaves)


def owned_of(state, n):
    sl = (Ellipsis,) + tuple(slice(G, G + m) for m in n)
    return BSSNVariables(*(np.asarray(leaf)[sl] for leaf in state))


def load_case(name):
    data = load_golden(f"fmr_{name}")
    hierarchy = hierarchy_of(data)
    root = root_params_of(data)
    params, shapes = ofmr.patch_parameters(root, tuple(int(v) for v in data["root_shape"]), hierarchy)
    count = len(shapes)
    initial = tuple(padded_from_owned(s, n) for s, n in zip(owned_states(data, "initial", count), shapes))
    initial = ofmr.prepare(initial, params, shapes, hierarchy, project=False)
    return data, hierarchy, params, shapes, initial
