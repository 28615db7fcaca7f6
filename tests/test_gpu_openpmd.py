"""Output staging: owned boxes gathered on the device equal the reference's
host-side slicing (diagnostics/openpmd.py:51-71, 254-285) bit for bit."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def op(cuda, native):
    from jax_bssn_gb300.diagnostics import openpmd
    return openpmd


def _fields(rng, shape, nvec=2, nscalar=3):
    out = {}
    for i in range(nscalar):
        out[f"s{i}"] = rng.standard_normal(shape)
    for i in range(nvec):
        out[f"v{i}"] = tuple(rng.standard_normal(shape) for _ in range(3))
    return out


def _strip(a, g):
    return a[tuple(slice(w, a.shape[d] - w) for d, w in enumerate(g))]


@pytest.mark.parametrize("ghost", [0, 2, (1, 2, 3)])
def test_stage_output_fields(op, ghost):
    rng = np.random.default_rng(3)
    fields = _fields(rng, (11, 14, 17))
    staged = op.stage_output_fields(fields, ghost)
    g = (ghost,) * 3 if isinstance(ghost, int) else ghost
    for name, field in fields.items():
        if isinstance(field, tuple):
            for got, want in zip(staged[name], field):
                assert isinstance(got, np.ndarray)
                np.testing.assert_array_equal(got, _strip(want, g))
        else:
            np.testing.assert_array_equal(staged[name], _strip(field, g))


def test_strip_ghost_cells_on_device_and_many_boxes(op):
    rng = np.random.default_rng(4)
    fields = _fields(rng, (9, 10, 12), nvec=12, nscalar=2)   # 38 boxes: two gather launches
    dev = {k: (tuple(torch.as_tensor(c, device="cuda") for c in v) if isinstance(v, tuple)
               else torch.as_tensor(v, device="cuda")) for k, v in fields.items()}
    out = op.strip_ghost_cells(dev, 2)
    for name, field in fields.items():
        got = out[name] if isinstance(field, tuple) else (out[name],)
        want = field if isinstance(field, tuple) else (field,)
        for a, b in zip(got, want):
            assert a.is_cuda
            np.testing.assert_array_equal(a.cpu().numpy(), _strip(b, (2, 2, 2)))


def test_tiled_output_fields(op):
    from jax_bssn_gb300.fmr import TileLayout
    layout = TileLayout((13, 9, 21))
    rng = np.random.default_rng(5)
    alloc = (1, 1, 1) + tuple(layout.allocated_shape)
    fields = {"W": rng.standard_normal(alloc), "shift": tuple(rng.standard_normal(alloc) for _ in range(3))}
    out = op.tiled_output_fields(fields, layout)
    g = layout.guard_cells
    np.testing.assert_array_equal(out["W"], fields["W"][0, 0, 0, g:g + 13, g:g + 9, g:g + 21])
    for a, b in zip(out["shift"], fields["shift"]):
        np.testing.assert_array_equal(a, b[0, 0, 0, g:g + 13, g:g + 9, g:g + 21])
    with pytest.raises(ValueError, match="does not match its tile layout"):
        op.tiled_output_fields({"W": rng.standard_normal((5, 5, 5))}, layout)


def test_staging_errors(op):
    with pytest.raises(ValueError, match="non-negative"):
        op.stage_output_fields({"a": np.zeros((4, 4, 4))}, -1)
    with pytest.raises(ValueError, match="empty axis"):
        op.stage_output_fields({"a": np.zeros((4, 4, 4))}, 2)


def test_empty_field_map(op):
    assert op.stage_output_fields({}, 2) == {}
