"""Parity at the benchmarked sizes, against oracle pins (tests/golden/pin_*.npz).

The benchmark's three evolution workloads are far larger than the golden
cases, and the oracle needs minutes per step there, so
tests/golden/make_bench_pins.py ran it once and stored, per snapshot and leaf,
the values on a sample set (every sample of the four outer rows at each face
and a lattice) plus whole-field statistics.  Here the CUDA path runs the same
configurations through the public calls and is compared on those samples:

  Teukolsky 128^3 (rk4_step, JAX_BSSN/evolution/time_evolve.py:144-217):
      1 step within 1e-12 and 10 steps within 1e-10 per leaf;
  nested FMR 96^3 + 65^3 + 49^3 (fmr_rk4_step, JAX_BSSN/fmr/tiled.py:182-209):
      1 step within 1e-12 per leaf and patch;
  axisymmetric punctures 256x512 (axisymmetric_rk4_step,
      JAX_BSSN/cartoon/axisymmetry/evolution.py:40-65): 1 step within 1e-12.

Error metric: max over the samples of |cuda - oracle| divided by max |oracle|
over the whole leaf (the parity tests' norm-relative metric, evaluated on the
sample set).  The whole-field sums are compared as well.
"""

import numpy as np
import pytest

from .helpers import LEAVES, GOLDEN

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-12
LONG_TOL = 1e-10


def _pin(name):
    path = GOLDEN / f"pin_{name}.npz"
    with np.load(path) as data:
        return {k: data[k] for k in data.files}


def _host(a):
    return a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)


def _errors(state, data, prefix, sets):
    ix = np.ix_(*sets)
    out = {}
    for leaf, value in zip(LEAVES, state):
        a = _host(value)
        got = a[(Ellipsis,) + ix]
        ref = data[f"{prefix}.{leaf}.samples"]
        scale = max(float(np.max(data[f"{prefix}.{leaf}.max"])), 1e-300)
        err = float(np.max(np.abs(got - ref))) / scale
        # whole-field sums: a wrong value anywhere moves them
        flat = a.reshape(a.shape[:-3] + (-1,))
        count = flat.shape[-1]
        sums = np.sum(flat, axis=-1)
        sum_err = float(np.max(np.abs(sums - data[f"{prefix}.{leaf}.sum"]))) / (scale * count)
        out[leaf] = max(err, sum_err)
    return out


def _report(tag, err):
    print(tag, {k: f"{v:.1e}" for k, v in err.items()})


def _triangles(state, data, prefix, sets):
    """Samples error of At's upper triangle (i <= j, the independent
    components both codes evolve) and of its lower triangle."""
    ix = np.ix_(*sets)
    a = _host(state.traceless_K)[(Ellipsis,) + ix]
    ref = data[f"{prefix}.traceless_K.samples"]
    scale = float(np.max(data[f"{prefix}.traceless_K.max"]))
    upper = max(float(np.max(np.abs(a[i, j] - ref[i, j]))) for i in range(3) for j in range(i, 3)) / scale
    lower = max(float(np.max(np.abs(a[i, j] - ref[i, j]))) for i in range(3) for j in range(i)) / scale
    return upper, lower


def test_teukolsky128_one_and_ten_steps(cuda, native):
    from jax_bssn_gb300.evolution import time_evolve as te
    from jax_bssn_gb300.initial_data import teukolsky_config
    data = _pin("teukolsky128")
    sets = tuple(data[f"axis{a}"] for a in range(3))
    state, params = teukolsky_config(n=128)
    init = _errors(state, data, "initial", sets)
    assert max(init.values()) < 1e-14, init          # same initial data as the pin
    one = te.rk4_step(state, params)
    e1 = _errors(one, data, "rk4_1", sets)
    _report("teukolsky128 1 step", e1)
    print("teukolsky128 1 step At upper/lower triangle", _triangles(one, data, "rk4_1", sets))
    assert max(e1.values()) < STEP_TOL
    ten = te.rk4_steps(one, params, 9)
    e10 = _errors(ten, data, "rk4_10", sets)
    _report("teukolsky128 10 steps", e10)
    assert max(e10.values()) < LONG_TOL


def test_fmr96_one_step(cuda, native):
    from jax_bssn_gb300.fmr import fmr_rk4_step, initialize_tiled_fmr
    from jax_bssn_gb300.initial_data import fmr_linear_wave_hierarchy, fmr_linear_wave_root
    from jax_bssn_gb300.bssn.variables import BSSNVariables
    data = _pin("fmr96")
    hierarchy = fmr_linear_wave_hierarchy(96)
    # the wave's stored x-profiles, broadcast over each patch (the same bits
    # the pin started from)
    profiles = [[data[f"profile.{k}.{leaf}"] for leaf in LEAVES] for k in range(3)]
    patch = iter(range(3))

    def initial(coordinates, local_params):
        shape = np.broadcast_shapes(*(np.shape(c) for c in coordinates))
        return BSSNVariables(*(np.broadcast_to(a, a.shape[:-3] + shape) for a in profiles[next(patch)]))
    states, parameters, layouts = initialize_tiled_fmr(initial, fmr_linear_wave_root(96), (96,) * 3, hierarchy)
    stepped = fmr_rk4_step(states, parameters, hierarchy, layouts=layouts)
    for k, (before, after, layout) in enumerate(zip(states, stepped, layouts)):
        n = layout.active_shape
        sets = tuple(data[f"patch{k}.axis{a}"] for a in range(3))
        owned = (Ellipsis,) + tuple(slice(4, 4 + m) for m in n)

        def own(s):
            return tuple(_host(leaf).reshape(leaf.shape[:-6] + leaf.shape[-3:])[owned] for leaf in s)
        init = _errors(own(before), data, f"initial.{k}", sets)
        assert max(init.values()) < 1e-14, (k, init)
        e1 = _errors(own(after), data, f"rk4_1.{k}", sets)
        _report(f"fmr96 patch {k} 1 step", e1)
        assert max(e1.values()) < STEP_TOL, k


def test_axisymmetric256_one_step(cuda, native):
    from jax_bssn_gb300.cartoon.axisymmetry import axisymmetric_rk4_step
    from jax_bssn_gb300.initial_data import brill_lindquist_config
    data = _pin("axisymmetric256")
    sets = tuple(data[f"axis{a}"] for a in range(3))
    state, params = brill_lindquist_config(num_radial_points=256, r_max=8.0)
    init = _errors(state, data, "initial", sets)
    assert max(init.values()) < 1e-14, init
    one = axisymmetric_rk4_step(state, params)
    e1 = _errors(one, data, "rk4_1", sets)
    _report("axisymmetric256 1 step", e1)
    assert max(e1.values()) < STEP_TOL
