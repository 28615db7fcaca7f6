"""The FMR oracle against the reference's tiled FMR run (goldens)."""

import json

import numpy as np
import pytest

from oracle import fmr as ofmr
from oracle.state import BSSNVariables

from .fmr_helpers import load_case, owned_of, owned_states
from .helpers import LEAVES, field_errors, worst

CASES = ("three_level_mad", "sommerfeld_kappa", "siblings_no_mad")


@pytest.fixture(scope="module", params=CASES)
def case(request):
    return (request.param,) + load_case(request.param)


def test_stage_rhs_and_prolonged_shell(case):
    name, data, hierarchy, params, shapes, initial = case
    prepared, rhs = ofmr.stage(initial, params, shapes, hierarchy)
    expect = owned_states(data, "stage1_rhs", len(shapes))
    for p, n in enumerate(shapes):
        assert worst(field_errors(owned_of(rhs[p], n), expect[p])) == 0.0, (name, p)
    last = len(shapes) - 1
    shell = BSSNVariables(*(data[f"stage1_prepared.{last}.{leaf}"] for leaf in LEAVES))
    assert worst(field_errors(prepared[last], shell)) == 0.0


def test_rk4_steps_and_norms(case):
    name, data, hierarchy, params, shapes, initial = case
    one = ofmr.rk4_step(initial, params, shapes, hierarchy)
    expect = owned_states(data, "rk4_1", len(shapes))
    for p, n in enumerate(shapes):
        assert worst(field_errors(owned_of(one[p], n), expect[p])) == 0.0, (name, p)
    last = len(shapes) - 1
    padded = BSSNVariables(*(data[f"rk4_1_padded.{last}.{leaf}"] for leaf in LEAVES))
    assert worst(field_errors(one[last], padded)) == 0.0
    two = ofmr.rk4_step(one, params, shapes, hierarchy)
    expect = owned_states(data, "rk4_2", len(shapes))
    for p, n in enumerate(shapes):
        assert worst(field_errors(owned_of(two[p], n), expect[p])) == 0.0, (name, p)
    norms = ofmr.constraint_norms(two, params, shapes, hierarchy)
    ref = json.loads(str(data["norms"]))
    for key, value in ref.items():
        assert norms[key] == pytest.approx(value, rel=1e-12, abs=1e-300), key
