"""Physical wave fields and composite diagnostics (mirrors JAX_BSSN/diagnostics/waves.py).

``h_plus`` runs one kernel over the reference layout (bit-identical to the
float64 reference), ``diagnostic_fields`` adds the constraint kernel's H and
M_i, and ``composite_wave_diagnostics`` reduces each level of a patch tree on
the device (``bssn_wave_norm_sums``) over the vertices its children do not
cover, then combines the levels' sums on the host.
"""

from __future__ import annotations

import ctypes
import math

import torch

from .. import _device, _native
from ..bssn.constraints import compute_all_constraints
from ..fmr.refinement import fine_active_view, hierarchy_parents


def h_plus(variables):
    """The physical plus-polarised metric perturbation (waves.py:11-20)."""
    lib = _native.load()
    state, host = _device.device_state(variables)
    shape = _device.spatial_shape(state)
    out = torch.empty(shape, dtype=torch.float64, device=state.lapse.device)
    _native.check(lib.bssn_h_plus(_device.fields_struct(state), _device.shape3(shape), out.data_ptr(),
                                  _device.stream_handle()), "h_plus")
    return out.cpu().numpy() if host else out


def diagnostic_fields(variables, parameters):
    """Wave and BSSN constraint fields for one grid level (waves.py:23-39)."""
    state, host = _device.device_state(variables)
    c = compute_all_constraints(state, parameters)
    fields = {
        "h_plus": h_plus(state),
        "lapse": state.lapse,
        "shift": tuple(state.shift[i] for i in range(3)),
        "K": state.trace_K,
        "W": state.conformal_factor,
        "hamiltonian_constraint": c.hamiltonian,
        "momentum_constraint": tuple(c.momentum[i] for i in range(3)),
    }
    if host:
        fields = {k: (tuple(x.cpu().numpy() for x in v) if isinstance(v, tuple) else v.cpu().numpy())
                  for k, v in fields.items()}
    return fields


def _field(value, device) -> torch.Tensor:
    return _device.as_device(value, tuple(value.shape), device, "diagnostic field").contiguous()


def composite_wave_diagnostics(level_fields, level_coordinates, hierarchy, time, amplitude, wavelength, *,
                               active_fields=False):
    """Point-count wave/constraint norms on uncovered vertices of a patch tree
    (waves.py:43-91)."""
    lib = _native.load()
    device = _device.require_cuda()
    parents = hierarchy_parents(hierarchy)
    ws = _device.workspace(lib.bssn_wave_norm_workspace_bytes(), device, tag="wave_norms")
    totals = torch.zeros((len(level_fields), 5), dtype=torch.float64, device=device)
    for level, (fields, coordinates) in enumerate(zip(level_fields, level_coordinates)):
        h, H = fields["h_plus"], fields["hamiltonian_constraint"]
        M = fields["momentum_constraint"]
        if level and not active_fields:
            spec = hierarchy.patches[level - 1]
            h, H, coordinates = (fine_active_view(x, spec) for x in (h, H, coordinates))
            M = tuple(fine_active_view(m, spec) for m in M)
        h, H, x = (_field(v, device) for v in (h, H, coordinates))
        M = torch.stack([_field(m, device) for m in M]).contiguous()
        shape = tuple(h.shape)
        if len(shape) != 3 or tuple(H.shape) != shape or tuple(x.shape) != shape or tuple(M.shape[1:]) != shape:
            raise ValueError("diagnostic fields and coordinates of a level must share one 3-D shape")
        boxes = []
        for child_index, parent in enumerate(parents[1:], start=1):
            if parent == level:
                child = hierarchy.patches[child_index - 1]
                boxes.extend(list(child.coarse_lo) + list(child.coarse_hi))
        covered = (ctypes.c_int32 * max(len(boxes), 1))(*boxes)
        _native.check(lib.bssn_wave_norm_sums(h.data_ptr(), x.data_ptr(), H.data_ptr(), M.data_ptr(),
                                              _device.shape3(shape), covered, len(boxes) // 6, float(time),
                                              float(amplitude), float(wavelength), totals[level].data_ptr(),
                                              ws.data_ptr(), ws.numel(), _device.stream_handle()),
                      "composite_wave_diagnostics")
    sums = totals.cpu().tolist()
    error_sum = sum(s[0] for s in sums)
    maximum = max((s[1] for s in sums), default=0.0)
    hamiltonian_sum = sum(s[2] for s in sums)
    momentum_sum = sum(s[3] for s in sums)
    point_count = int(round(sum(s[4] for s in sums)))
    rms = math.sqrt(error_sum / point_count)
    return {
        "composite_rms": rms,
        "composite_max": maximum,
        "composite_hamiltonian_l2": math.sqrt(hamiltonian_sum / point_count),
        "composite_momentum_l2": math.sqrt(momentum_sum / point_count),
        "coarse_rms": rms,
        "fine_rms": rms,
    }
