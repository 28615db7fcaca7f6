"""Device-resident evolution of one grid in the padded patch layout.

The drop-in ``rk4_step`` converts the seven reference leaves to the kernels'
working layout on every call.  ``PatchEvolution`` keeps the state resident
instead -- 21 independent float64 components, each a padded
(nx+2G)(ny+2G)(nz+2G) block -- so a run of steps touches only HBM.  It is the
same algorithm as ``rk4_step`` repeated (JAX_BSSN/evolution/time_evolve.py:144-217)
on a periodic/Sommerfeld grid.
"""

from __future__ import annotations

import torch

from .. import _device, _native
from .._graph import GraphSteps
from ..bssn.variables import BSSNParameters, BSSNVariables

NCOMP = 21


class PatchEvolution(GraphSteps):
    def __init__(self, vars: BSSNVariables, params: BSSNParameters, ghost: int = 4, precision: str | None = None):
        if params.guard_cells or params.owned_shape is not None:
            raise ValueError("PatchEvolution evolves a whole unpadded grid (guard_cells=0, owned_shape=None)")
        self.lib = _native.load()
        state, _ = _device.device_state(vars)
        self.device = state.lapse.device
        self.shape = _device.spatial_shape(state)
        self.params = params
        self.patch = _native.BssnPatch()
        for d in range(3):
            self.patch.n[d] = self.shape[d]
        self.patch.ghost = int(ghost)
        self.cparams = _device.to_params(params, precision)
        values = self.lib.bssn_patch_values(self.patch)
        if values == 0:
            raise ValueError("invalid patch description")
        self.padded = tuple(n + 2 * ghost for n in self.shape)
        self.u = torch.zeros(values, dtype=torch.float64, device=self.device)
        nbytes = self.lib.bssn_patch_workspace_bytes(self.patch, self.cparams)
        self.ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        _native.check(self.lib.bssn_patch_import(_device.fields_struct(state), self.u.data_ptr(), self.patch,
                                                 _device.stream_handle()), "bssn_patch_import")

    def _advance(self, steps: int) -> None:
        _native.check(self.lib.bssn_patch_rk4(self.u.data_ptr(), self.patch, self.cparams, int(steps),
                                              self.ws.data_ptr(), self.ws.numel(), _device.stream_handle()),
                      "bssn_patch_rk4")

    def tune(self, margin: float = 0.98) -> str:
        """Autotune the RHS launch shapes for this grid and arithmetic form
        (later steps and graph captures use them; results are unchanged).  A
        shape changes only when it is faster than ``margin`` x the current one."""
        return _native.tune_launch_shapes(self.u.data_ptr(), self.shape, 1, self.cparams, self.device, self.ws,
                                          margin)

    def state(self) -> BSSNVariables:
        out = _device.empty_state(self.shape, self.device)
        _native.check(self.lib.bssn_patch_export(self.u.data_ptr(), _device.fields_struct(out), self.patch,
                                                 _device.stream_handle()), "bssn_patch_export")
        return out

    def components(self) -> torch.Tensor:
        """View of the resident state as (21, nx+2G, ny+2G, nz+2G)."""
        return self.u.view(NCOMP, *self.padded)

    def nonfinite_count(self) -> int:
        flag = torch.zeros(1, dtype=torch.int32, device=self.device)
        _native.check(self.lib.bssn_patch_check_finite(self.u.data_ptr(), self.patch, flag.data_ptr(),
                                                       _device.stream_handle()), "bssn_patch_check_finite")
        return int(flag.item())


class NonFiniteStateError(FloatingPointError):
    """A monitored evolution found NaN or infinite values; ``steps_done`` RK4
    steps had completed before the check that found them."""

    def __init__(self, message: str, steps_done: int):
        super().__init__(message)
        self.steps_done = steps_done


class BatchEvolution(GraphSteps):
    """Many independent instances of one grid, advanced by the same launches.

    Every instance has the same shape and parameters (a seed ensemble, a set
    of replicas); each is the reference's ``rk4_step`` repeated on its own
    state.  The resident layout is [component][instance][padded block], so a
    kernel launch covers every instance and one captured graph advances them
    all.  Results equal separate ``PatchEvolution`` runs bit for bit.
    """

    def __init__(self, states, params: BSSNParameters, ghost: int = 4, precision: str | None = None):
        states = list(states)
        if not states:
            raise ValueError("BatchEvolution needs at least one instance")
        if params.guard_cells or params.owned_shape is not None:
            raise ValueError("BatchEvolution evolves whole unpadded grids (guard_cells=0, owned_shape=None)")
        self.lib = _native.load()
        first, _ = _device.device_state(states[0])
        self.device = first.lapse.device
        self.shape = _device.spatial_shape(first)
        self.params = params
        self.instances = len(states)
        self.patch = _native.BssnPatch()
        for d in range(3):
            self.patch.n[d] = self.shape[d]
        self.patch.ghost = int(ghost)
        self.cparams = _device.to_params(params, precision)
        values = self.lib.bssn_batch_values(self.patch, self.instances)
        if values == 0:
            raise ValueError("invalid patch description")
        self.padded = tuple(n + 2 * ghost for n in self.shape)
        self.u = torch.zeros(values, dtype=torch.float64, device=self.device)
        nbytes = self.lib.bssn_batch_workspace_bytes(self.patch, self.instances, self.cparams)
        self.ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        for i, vars in enumerate(states):
            state, _ = _device.device_state(vars)
            if _device.spatial_shape(state) != self.shape:
                raise ValueError("every instance must have the same grid shape")
            _native.check(self.lib.bssn_batch_import(_device.fields_struct(state), self.u.data_ptr(), self.patch,
                                                     self.instances, i, _device.stream_handle()),
                          "bssn_batch_import")

    def _advance(self, steps: int) -> None:
        _native.check(self.lib.bssn_batch_rk4(self.u.data_ptr(), self.patch, self.instances, self.cparams,
                                              int(steps), self.ws.data_ptr(), self.ws.numel(),
                                              _device.stream_handle()), "bssn_batch_rk4")

    def state(self, instance: int = 0) -> BSSNVariables:
        out = _device.empty_state(self.shape, self.device)
        _native.check(self.lib.bssn_batch_export(self.u.data_ptr(), _device.fields_struct(out), self.patch,
                                                 self.instances, int(instance), _device.stream_handle()),
                      "bssn_batch_export")
        return out

    def tune(self, margin: float = 0.98) -> str:
        """Autotune the RHS launch shapes for this batch and arithmetic form."""
        return _native.tune_launch_shapes(self.u.data_ptr(), self.shape, self.instances, self.cparams, self.device,
                                          self.ws, margin)

    def step_monitored(self, steps: int, check_every: int = 1) -> int:
        """``steps`` RK4 steps, counting non-finite values before the first and
        every ``check_every`` steps; raises ``NonFiniteStateError`` (carrying
        the steps completed) at the first check that finds any."""
        import ctypes
        counter = torch.zeros(1, dtype=torch.int32, device=self.device)
        done = ctypes.c_int32(0)
        status = self.lib.bssn_batch_rk4_monitored(self.u.data_ptr(), self.patch, self.instances, self.cparams,
                                                   int(steps), int(check_every), counter.data_ptr(),
                                                   ctypes.byref(done), self.ws.data_ptr(), self.ws.numel(),
                                                   _device.stream_handle())
        if status == _native.BSSN_ERR_NONFINITE:
            raise NonFiniteStateError(_native.last_error(), done.value)
        _native.check(status, "bssn_batch_rk4_monitored")
        return done.value

    def states(self) -> list:
        return [self.state(i) for i in range(self.instances)]

    def components(self) -> torch.Tensor:
        """View of the resident state as (21, instances, nx+2G, ny+2G, nz+2G)."""
        return self.u.view(NCOMP, self.instances, *self.padded)

    def nonfinite_count(self) -> int:
        flag = torch.zeros(1, dtype=torch.int32, device=self.device)
        _native.check(self.lib.bssn_batch_check_finite(self.u.data_ptr(), self.patch, self.instances,
                                                       flag.data_ptr(), _device.stream_handle()),
                      "bssn_batch_check_finite")
        return int(flag.item())
