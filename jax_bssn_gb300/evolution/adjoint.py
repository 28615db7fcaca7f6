"""Reverse-mode differentiation of BSSN evolutions on the GPU.

The reference has no adjoint of its own: a gradient through its rk4_step
(JAX_BSSN/evolution/time_evolve.py:144-217) would be jax.grad over XLA's
reverse mode.  Here the vector-Jacobian products are CUDA kernels
(``bssn_adjoint.cu``): the generated reverse sweep of the pointwise BSSN
algebra, transposed finite-difference stencils, and the reverse of the
projection and RK4 combination, with sqrt(N) checkpointing of the state.

States are batches of independent instances in component form: a float64
tensor (21, instances, nx, ny, nz) of the independent components in the
order gt_xx gt_xy gt_xz gt_yy gt_yz gt_zz, W, At_xx ... At_zz, K, Gt^i, alpha,
beta^i.  ``components`` / ``leaves`` convert one instance from and to the
reference's seven leaves.  Gradients are taken with respect to these 21
components; for a symmetric tensor the off-diagonal component's gradient is
the sum over both halves of a full 3x3 array.

Scope: each axis periodic or closed by Sommerfeld faces at both ends (the
one-sided closure rows and the radial face condition are transposed as well);
kappa = 0, no matter sources, FP64 arithmetic.
"""

from __future__ import annotations

import torch

from .. import _device, _native
from ..bssn.variables import BSSNParameters, BSSNVariables

NCOMP = 21
_PAIRS = ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))


def components(state: BSSNVariables) -> torch.Tensor:
    """Seven reference leaves -> (21, nx, ny, nz); tensors from their upper triangle."""
    g, W, A, K, G, al, b = (torch.as_tensor(f, dtype=torch.float64) for f in state)
    parts = [g[i, j] for i, j in _PAIRS] + [W] + [A[i, j] for i, j in _PAIRS] + [K] + [G[i] for i in range(3)]
    parts += [al] + [b[i] for i in range(3)]
    return torch.stack(parts)


def leaves(u: torch.Tensor) -> BSSNVariables:
    """(21, nx, ny, nz) -> the seven reference leaves (symmetric tensors filled)."""
    def sym(block):
        rows = [[None] * 3 for _ in range(3)]
        for c, (i, j) in enumerate(_PAIRS):
            rows[i][j] = rows[j][i] = block[c]
        return torch.stack([torch.stack(r) for r in rows])
    return BSSNVariables(sym(u[0:6]), u[6], sym(u[7:13]), u[13], u[14:17], u[17], u[18:21])


def _validate(params: BSSNParameters) -> None:
    faces = tuple(int(f) for f in (params.xl_bc, params.xr_bc, params.yl_bc, params.yr_bc, params.zl_bc, params.zr_bc))
    if any(f not in (0, 1) for f in faces) or any(faces[2 * d] != faces[2 * d + 1] for d in range(3)):
        raise ValueError("the adjoint needs both faces of each axis periodic (code 0) or both Sommerfeld (code 1)")
    if float(params.kappa) != 0.0:
        raise ValueError("the adjoint needs kappa = 0")
    if params.guard_cells or params.owned_shape is not None:
        raise ValueError("the adjoint evolves whole unpadded grids (guard_cells=0, owned_shape=None)")


class _Batch:
    """Padded batch buffers of one (shape, instances, params) configuration."""

    def __init__(self, shape, instances, params, device, ghost=4):
        _validate(params)
        self.lib = _native.load()
        self.shape = tuple(int(n) for n in shape)
        self.instances = int(instances)
        self.ghost = ghost
        self.device = device
        self.patch = _native.BssnPatch()
        for d in range(3):
            self.patch.n[d] = self.shape[d]
        self.patch.ghost = ghost
        self.cparams = _device.to_params(params, "fp64")
        self.padded = tuple(n + 2 * ghost for n in self.shape)
        self.values = self.lib.bssn_batch_values(self.patch, self.instances)
        if self.values == 0:
            raise ValueError("invalid patch description")

    def empty(self) -> torch.Tensor:
        return torch.zeros(self.values, dtype=torch.float64, device=self.device)

    def owned(self, buf: torch.Tensor) -> torch.Tensor:
        g = self.ghost
        view = buf.view(NCOMP, self.instances, *self.padded)
        return view[:, :, g:g + self.shape[0], g:g + self.shape[1], g:g + self.shape[2]]

    def load(self, u: torch.Tensor) -> torch.Tensor:
        buf = self.empty()
        self.owned(buf).copy_(u)
        return buf


def _batch_for(u: torch.Tensor, params: BSSNParameters) -> _Batch:
    if u.dim() != 5 or u.shape[0] != NCOMP:
        raise ValueError("expected a (21, instances, nx, ny, nz) component tensor")
    if u.dtype != torch.float64 or u.device.type != "cuda":
        raise ValueError("expected a float64 CUDA tensor")
    return _Batch(u.shape[2:], u.shape[1], params, u.device)


def rhs_vjp(u: torch.Tensor, rhs_adjoint: torch.Tensor, params: BSSNParameters) -> torch.Tensor:
    """(d RHS / d u)^T rhs_adjoint for a component batch u (compute_bssn_rhs,
    JAX_BSSN/evolution/time_evolve.py:41-57)."""
    B = _batch_for(u, params)
    state, kbar, out = B.load(u), B.load(rhs_adjoint), B.empty()
    ws = torch.empty(B.lib.bssn_rhs_vjp_workspace_bytes(B.patch, B.instances), dtype=torch.uint8, device=B.device)
    _native.check(B.lib.bssn_rhs_vjp(state.data_ptr(), kbar.data_ptr(), out.data_ptr(), B.patch, B.instances,
                                     B.cparams, ws.data_ptr(), ws.numel(), _device.stream_handle()), "bssn_rhs_vjp")
    return B.owned(out).clone()


class CheckpointedEvolution:
    """`steps` RK4 steps of a component batch with sqrt(N) checkpoints kept
    for a later ``backward``.  ``segment`` (default ceil(sqrt(steps))) steps
    separate checkpoints.  ``store_stages`` sets what a re-run segment keeps:
    0 step-start states only (stages recomputed: two forward re-runs), 1 (or
    True) also the stage RHS values (one re-run), 2 also the stage states
    (one re-run, no stage replay; the most memory)."""

    def __init__(self, u0: torch.Tensor, params: BSSNParameters, steps: int, segment: int = 0,
                 store_stages: int = 1):
        self.B = _batch_for(u0, params)
        self.steps, self.segment, self.store = int(steps), int(segment), int(store_stages)
        if self.store not in (0, 1, 2):
            raise ValueError("store_stages must be 0, 1 or 2")
        if self.steps < 0:
            raise ValueError("steps must be non-negative")
        nbytes = self.B.lib.bssn_adjoint_workspace_bytes(self.B.patch, self.B.instances, self.B.cparams, self.steps,
                                                         self.segment, self.store)
        if nbytes == 0:
            raise ValueError(_native.last_error())
        self.ws = torch.empty(nbytes, dtype=torch.uint8, device=self.B.device)
        self.state = self.B.load(u0)
        self.forward_done = False

    def _args(self):
        return (self.B.patch, self.B.instances, self.B.cparams, self.steps, self.segment, self.store,
                self.ws.data_ptr(), self.ws.numel(), _device.stream_handle())

    def forward(self) -> torch.Tensor:
        """Advance in place and record checkpoints; returns the final owned state."""
        _native.check(self.B.lib.bssn_adjoint_forward(self.state.data_ptr(), *self._args()), "bssn_adjoint_forward")
        self.forward_done = True
        return self.B.owned(self.state)

    def backward(self, final_adjoint: torch.Tensor) -> torch.Tensor:
        """d loss / d initial state from d loss / d final state (once per forward)."""
        if not self.forward_done:
            raise RuntimeError("backward needs a recorded forward pass (one backward per forward)")
        adj = self.B.load(final_adjoint)
        _native.check(self.B.lib.bssn_adjoint_backward(adj.data_ptr(), *self._args()), "bssn_adjoint_backward")
        self.forward_done = False   # the backward pass reuses the recorded segment's memory
        return self.B.owned(adj).clone()


class RK4Evolve(torch.autograd.Function):
    """u_N = rk4_step^N(u_0) on a component batch, differentiable in u_0 by
    the adjoint kernels (torch.autograd.Function over the C ABI)."""

    @staticmethod
    def forward(ctx, u0, params, steps, segment=0, store_stages=1):
        run = CheckpointedEvolution(u0.detach(), params, steps, segment, store_stages)
        out = run.forward().clone()
        ctx.run = run
        return out

    @staticmethod
    def backward(ctx, grad_out):
        grad = ctx.run.backward(grad_out.contiguous())
        ctx.run = None
        return grad, None, None, None, None


def evolve(u0: torch.Tensor, params: BSSNParameters, steps: int, segment: int = 0,
           store_stages: int = 1) -> torch.Tensor:
    """Differentiable ``steps`` RK4 steps of a (21, instances, nx, ny, nz) batch."""
    return RK4Evolve.apply(u0, params, steps, segment, store_stages)
