"""The Cartoon C-ABI calls shared by the axisymmetric and spherical modules.

A compact state (seven leaves, spatial extent (Nx, 1, Nz) or (Nr, 1, 1)) is
converted once into the kernels' 21-component layout, handed to
``libbssn_gb300.so`` and converted back.  Results follow the caller: CUDA
tensors in, CUDA tensors out; host arrays in, NumPy out.
"""

from __future__ import annotations

import torch

from .. import _device, _native
from .._graph import GraphSteps
from ..bssn.constraints import ConstraintViolations
from ..bssn.variables import BSSNParameters, BSSNVariables

NCOMP = 21
SUPPORT = 9


def to_components(lib, state: BSSNVariables, shape) -> torch.Tensor:
    u = torch.empty(NCOMP * _device.prod(shape), dtype=torch.float64, device=state.lapse.device)
    _native.check(lib.bssn_fields_to_components(_device.fields_struct(state), u.data_ptr(), _device.shape3(shape),
                                                _device.stream_handle()), "bssn_fields_to_components")
    return u


def to_fields(lib, u: torch.Tensor, shape) -> BSSNVariables:
    out = _device.empty_state(shape, u.device)
    _native.check(lib.bssn_components_to_fields(u.data_ptr(), _device.fields_struct(out), _device.shape3(shape),
                                                _device.stream_handle()), "bssn_components_to_fields")
    return out


def _finish(state: BSSNVariables, host: bool):
    return _device.to_host(state) if host else state


def _prepare(vars: BSSNVariables):
    lib = _native.load()
    state, host = _device.device_state(vars)
    shape = _device.spatial_shape(state)
    return lib, state, host, shape


def workspace(lib, axi: bool, shape, cparams, device) -> torch.Tensor:
    nbytes = lib.bssn_cartoon_workspace_bytes(int(axi), _device.shape3(shape), cparams)
    if nbytes == 0:
        _native.check(_native.BSSN_ERR_INVALID, "bssn_cartoon_workspace_bytes")
    return _device.workspace(nbytes, device, tag="cartoon")


def fill_ghosts(vars: BSSNVariables, axi: bool):
    lib, state, host, shape = _prepare(vars)
    u = to_components(lib, state, shape)
    _native.check(lib.bssn_cartoon_fill_ghosts(int(axi), u.data_ptr(), _device.shape3(shape),
                                               _device.stream_handle()), "bssn_cartoon_fill_ghosts")
    return _finish(to_fields(lib, u, shape), host)


def reconstruct(vars: BSSNVariables, params: BSSNParameters, axi: bool):
    lib, state, host, shape = _prepare(vars)
    cparams = _device.to_params(params)
    u = to_components(lib, state, shape)
    sshape = (shape[0], SUPPORT, shape[2]) if axi else (shape[0], SUPPORT, SUPPORT)
    s = torch.empty(NCOMP * _device.prod(sshape), dtype=torch.float64, device=u.device)
    _native.check(lib.bssn_cartoon_reconstruct(int(axi), u.data_ptr(), s.data_ptr(), _device.shape3(shape),
                                               cparams, _device.stream_handle()), "bssn_cartoon_reconstruct")
    return _finish(to_fields(lib, s, sshape), host)


def rhs(vars: BSSNVariables, params: BSSNParameters, axi: bool):
    lib, state, host, shape = _prepare(vars)
    cparams = _device.to_params(params)
    u = to_components(lib, state, shape)
    k = torch.empty_like(u)
    ws = workspace(lib, axi, shape, cparams, u.device)
    _native.check(lib.bssn_cartoon_rhs(int(axi), u.data_ptr(), k.data_ptr(), _device.shape3(shape), cparams,
                                       ws.data_ptr(), ws.numel(), _device.stream_handle()), "bssn_cartoon_rhs")
    return _finish(to_fields(lib, k, shape), host)


def rk4(vars: BSSNVariables, params: BSSNParameters, axi: bool, steps: int = 1):
    lib, state, host, shape = _prepare(vars)
    cparams = _device.to_params(params)
    u = to_components(lib, state, shape)
    ws = workspace(lib, axi, shape, cparams, u.device)
    _native.check(lib.bssn_cartoon_rk4_step(int(axi), u.data_ptr(), _device.shape3(shape), cparams, int(steps),
                                            ws.data_ptr(), ws.numel(), _device.stream_handle()),
                  "bssn_cartoon_rk4_step")
    return _finish(to_fields(lib, u, shape), host)


def constraints(vars: BSSNVariables, params: BSSNParameters, axi: bool) -> ConstraintViolations:
    lib, state, host, shape = _prepare(vars)
    cparams = _device.to_params(params)
    u = to_components(lib, state, shape)
    ws = workspace(lib, axi, shape, cparams, u.device)
    out = torch.empty((9,) + tuple(shape), dtype=torch.float64, device=u.device)
    _native.check(lib.bssn_cartoon_constraints(int(axi), u.data_ptr(), _device.shape3(shape), cparams,
                                               out.data_ptr(), ws.data_ptr(), ws.numel(), _device.stream_handle()),
                  "bssn_cartoon_constraints")
    v = ConstraintViolations(out[0], out[1:4], out[4], out[5], out[6:9])
    if host:
        v = ConstraintViolations(*(t.cpu().numpy() for t in v))
    return v


class CartoonEvolution(GraphSteps):
    """A compact Cartoon state kept resident in the 21-component layout.

    ``step(n)`` runs n classical RK4 steps (one C-ABI call) with no layout
    conversion; ``state()`` converts back to the seven leaves.
    """

    def __init__(self, vars: BSSNVariables, params: BSSNParameters, axisymmetric: bool,
                 precision: str | None = None):
        self.lib, state, _, self.shape = _prepare(vars)
        self.axi = bool(axisymmetric)
        self.params = params
        self.cparams = _device.to_params(params, precision)
        self.device = state.lapse.device
        self.u = to_components(self.lib, state, self.shape)
        nbytes = self.lib.bssn_cartoon_workspace_bytes(int(self.axi), _device.shape3(self.shape), self.cparams)
        if nbytes == 0:
            _native.check(_native.BSSN_ERR_INVALID, "bssn_cartoon_workspace_bytes")
        self.ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)

    def _advance(self, steps: int) -> None:
        _native.check(self.lib.bssn_cartoon_rk4_step(int(self.axi), self.u.data_ptr(), _device.shape3(self.shape),
                                                     self.cparams, int(steps), self.ws.data_ptr(), self.ws.numel(),
                                                     _device.stream_handle()), "bssn_cartoon_rk4_step")

    def state(self) -> BSSNVariables:
        return to_fields(self.lib, self.u, self.shape)

    def components(self) -> torch.Tensor:
        """View of the resident state as (21, Nx, 1, Nz)."""
        return self.u.view(NCOMP, *self.shape)

    def constraints(self) -> ConstraintViolations:
        out = torch.empty((9,) + tuple(self.shape), dtype=torch.float64, device=self.device)
        _native.check(self.lib.bssn_cartoon_constraints(int(self.axi), self.u.data_ptr(), _device.shape3(self.shape),
                                                        self.cparams, out.data_ptr(), self.ws.data_ptr(),
                                                        self.ws.numel(), _device.stream_handle()),
                      "bssn_cartoon_constraints")
        return ConstraintViolations(out[0], out[1:4], out[4], out[5], out[6:9])
