"""Oracle pins at the benchmarked sizes, for the GPU parity tests.

    PYTHONPATH=. python tests/golden/make_bench_pins.py teukolsky128
    PYTHONPATH=. python tests/golden/make_bench_pins.py fmr96
    PYTHONPATH=. python tests/golden/make_bench_pins.py axisymmetric256

Cases (the initial data come from ``jax_bssn_gb300.initial_data``, the same
host generator the benchmark uses, whose Teukolsky and Brill-Lindquist data
are built from IEEE-rounded operations only and so are the same bits on every
host; the evolution is the oracle, which the CPU tests pin bit for bit to
goldens of the reference source):

  teukolsky128     linearised Teukolsky quadrupole wave, 128^3 vertex grid over
                   [-4,4]^3, Sommerfeld faces, 1+log + Gamma driver: states
                   after 1 and 10 RK4 steps
  fmr96            linear wave (A=1e-8, lambda=4) through the 3-level nested
                   hierarchy, root 96^3, level 1 65^3, level 2 49^3: owned
                   states of every patch after 1 stage-synchronous RK4 step;
                   the wave's exact x-profiles are stored too (its K is second
                   order in the amplitude, ~1e-16, so its bits depend on the
                   host's sin/cos/pow: the GPU test starts from these)
  axisymmetric256  Brill-Lindquist punctures on the 260x1x512 compact Cartoon
                   plane (dx=1/32): compact state after 1 RK4 step

Full states (hundreds of MB at these sizes) are too large to commit, so each
snapshot keeps, per leaf and component, statistics of the whole field (max
|u|, sum, sum of squares) and the values on a sample set: the product of
per-axis index sets holding the four outer rows at each end of the axis (the
closure and face rows) and a regular lattice.
"""

from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LEAVES = ("conformal_metric", "conformal_factor", "traceless_K", "trace_K",
          "conformal_connection", "lapse", "shift")


def axis_samples(n: int, stride: int) -> np.ndarray:
    """Sample indices along one axis: the four outer rows at each end and a
    lattice of the given stride (ends included)."""
    edge = list(range(min(4, n))) + list(range(max(n - 4, 0), n))
    return np.unique(np.array(edge + list(range(0, n, stride)) + [n - 1], dtype=np.int64))


def sample_sets(shape, strides):
    return tuple(axis_samples(n, s) for n, s in zip(shape, strides))


def snapshot(state, sets) -> dict:
    """Statistics of every leaf component and its values on the sample set."""
    ix = np.ix_(*sets)
    out = {}
    for leaf, a in zip(LEAVES, state):
        a = np.asarray(a, dtype=np.float64)
        flat = a.reshape(a.shape[:-3] + (-1,))
        out[f"{leaf}.max"] = np.max(np.abs(flat), axis=-1)
        out[f"{leaf}.sum"] = np.sum(flat, axis=-1)
        out[f"{leaf}.sumsq"] = np.sum(flat * flat, axis=-1)
        out[f"{leaf}.samples"] = a[(Ellipsis,) + ix]
    return out


def _save(name: str, meta: dict, sets, snaps: dict) -> None:
    arrays = {"meta": np.array(json.dumps(meta))}
    for axis, s in enumerate(sets):
        arrays[f"axis{axis}"] = s
    for tag, snap in snaps.items():
        for key, value in snap.items():
            arrays[f"{tag}.{key}"] = value
    np.savez_compressed(HERE / f"pin_{name}.npz", **arrays)


def teukolsky128() -> None:
    from jax_bssn_gb300.initial_data import teukolsky_config
    from oracle import bssn as ob
    from oracle.state import BSSNParameters as OP, BSSNVariables as OV
    state, params = teukolsky_config(n=128)
    s, p = OV(*(np.asarray(f) for f in state)), OP(**params._asdict())
    sets = sample_sets((128,) * 3, (16,) * 3)
    snaps = {"initial": snapshot(s, sets)}
    for step in range(1, 11):
        t = time.time()
        s = ob.rk4_step(s, p)
        print(f"teukolsky128 step {step}: {time.time() - t:.1f} s", flush=True)
        if step in (1, 10):
            snaps[f"rk4_{step}"] = snapshot(s, sets)
    _save("teukolsky128", {"n": 128, "steps": [1, 10]}, sets, snaps)


def fmr96() -> None:
    from jax_bssn_gb300.initial_data import fmr_linear_wave_hierarchy, fmr_linear_wave_root, linear_wave_state
    from oracle import fmr as of
    from oracle.state import BSSNParameters as OP, BSSNVariables as OV
    root = 96
    h = fmr_linear_wave_hierarchy(root)
    oh = of.FMRHierarchySpec(tuple(of.FMRPatchSpec(s.coarse_lo, s.coarse_hi, parent=s.parent) for s in h.patches),
                             use_mad=h.use_mad)
    params, shapes = of.patch_parameters(OP(**fmr_linear_wave_root(root)._asdict()), (root,) * 3, oh)
    # The wave depends on x only: its exact x-profiles (kept in the pin, so the
    # GPU test starts from the same bits whatever the host's libm) broadcast
    # over y and z give every patch's owned state.
    profiles = []
    states = []
    for p, n in zip(params, shapes):
        X = p.x_min + p.dx * (np.arange(n[0], dtype=np.float64) + 0.0)
        flat = X[:, None, None]
        profile = linear_wave_state(flat, np.zeros_like(flat), np.zeros_like(flat), 1e-8, 4.0)
        profiles.append(profile)
        leaves = []
        for leaf in profile:
            leaf = np.asarray(leaf)
            lead = leaf.shape[:-3]
            full = np.zeros(lead + tuple(m + 2 * of.GUARD for m in n))
            full[(Ellipsis,) + tuple(slice(of.GUARD, of.GUARD + m) for m in n)] = np.broadcast_to(leaf, lead + n)
            leaves.append(full)
        states.append(OV(*leaves))
    states = of.prepare(tuple(states), params, shapes, oh, project=False)
    t = time.time()
    stepped = of.rk4_step(states, params, shapes, oh)
    print(f"fmr96 step: {time.time() - t:.1f} s", flush=True)
    G = of.GUARD
    snaps, all_sets = {}, []
    for k, (n, before, after) in enumerate(zip(shapes, states, stepped)):
        sets = sample_sets(n, (12,) * 3)
        all_sets.append(sets)
        owned = tuple(slice(G, G + m) for m in n)
        snaps[f"initial.{k}"] = snapshot(tuple(np.asarray(a)[(Ellipsis,) + owned] for a in before), sets)
        snaps[f"rk4_1.{k}"] = snapshot(tuple(np.asarray(a)[(Ellipsis,) + owned] for a in after), sets)
    arrays = {"meta": np.array(json.dumps({"root": root, "shapes": [list(n) for n in shapes]}))}
    for k, profile in enumerate(profiles):
        for leaf, value in zip(LEAVES, profile):
            arrays[f"profile.{k}.{leaf}"] = np.asarray(value)
    for k, sets in enumerate(all_sets):
        for axis, s in enumerate(sets):
            arrays[f"patch{k}.axis{axis}"] = s
    for tag, snap in snaps.items():
        for key, value in snap.items():
            arrays[f"{tag}.{key}"] = value
    np.savez_compressed(HERE / "pin_fmr96.npz", **arrays)


def axisymmetric256() -> None:
    from jax_bssn_gb300.initial_data import brill_lindquist_config
    from oracle import cartoon as oc
    from oracle.state import BSSNParameters as OP, BSSNVariables as OV
    state, params = brill_lindquist_config(num_radial_points=256, r_max=8.0)
    s, p = OV(*(np.asarray(f) for f in state)), OP(**params._asdict())
    shape = np.asarray(s.lapse).shape
    sets = sample_sets(shape, (8, 1, 8))
    snaps = {"initial": snapshot(s, sets)}
    t = time.time()
    s = oc.axi_rk4_step(s, p)
    print(f"axisymmetric256 step: {time.time() - t:.1f} s", flush=True)
    snaps["rk4_1"] = snapshot(s, sets)
    _save("axisymmetric256", {"shape": list(shape), "steps": [1]}, sets, snaps)


CASES = {"teukolsky128": teukolsky128, "fmr96": fmr96, "axisymmetric256": axisymmetric256}

if __name__ == "__main__":
    for name in sys.argv[1:] or list(CASES):
        CASES[name]()
