"""State and parameter containers mirroring the reference contract.

Follows JAX_BSSN/bssn/variables.py:8-46: seven leaves in a fixed order
(gamma_tilde (3,3,...), W, A_tilde (3,3,...), K, Gamma_tilde (3,...), alpha,
beta (3,...)) and a NamedTuple of scalar parameters.
"""

from typing import NamedTuple

import numpy as np


class BSSNVariables(NamedTuple):
    conformal_metric: np.ndarray
    conformal_factor: np.ndarray
    traceless_K: np.ndarray
    trace_K: np.ndarray
    conformal_connection: np.ndarray
    lapse: np.ndarray
    shift: np.ndarray


class BSSNParameters(NamedTuple):
    eta: float = 2.0
    kappa: float = 0.0
    nu: float = 0.002
    g: float = 0.75
    dx: float = 0.1
    dt: float = 0.001
    zero_shift: int = 0
    gauge: int = 0
    xl_bc: int = 0
    xr_bc: int = 0
    yl_bc: int = 0
    yr_bc: int = 0
    zl_bc: int = 0
    zr_bc: int = 0
    x_min: float = 0.0
    y_min: float = 0.0
    z_min: float = 0.0
    mad_q: float = 1.0
    guard_cells: int = 0
    owned_shape: tuple | None = None
    owned_faces: tuple = (True, True, True, True, True, True)
    reduced_axes: tuple | None = None


FACE_NAMES = ("xl_bc", "xr_bc", "yl_bc", "yr_bc", "zl_bc", "zr_bc")
LEAF_RANKS = (2, 0, 2, 0, 1, 0, 1)
SYM_PAIRS = ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))


def face_codes(params):
    return tuple(int(getattr(params, name)) for name in FACE_NAMES)


def pack_state(state):
    """Stack all 27 stored components along a new leading axis."""
    spatial = np.shape(state.conformal_factor)
    return np.concatenate([np.asarray(f).reshape((-1,) + spatial) for f in state])


def unpack_state(packed, spatial=None):
    spatial = packed.shape[1:] if spatial is None else spatial
    cuts = np.cumsum([0, 9, 1, 9, 1, 3, 1, 3])
    shapes = ((3, 3), (), (3, 3), (), (3,), (), (3,))
    return BSSNVariables(*(packed[a:b].reshape(s + tuple(spatial))
                           for a, b, s in zip(cuts[:-1], cuts[1:], shapes)))


def to_independent(state):
    """The 21 independent components (upper triangles) in kernel order."""
    g, W, A, K, G, a, b = (np.asarray(f) for f in state)
    comps = [g[i, j] for i, j in SYM_PAIRS] + [W] + [A[i, j] for i, j in SYM_PAIRS]
    comps += [K, G[0], G[1], G[2], a, b[0], b[1], b[2]]
    return np.stack(comps)


def from_independent(u):
    """Inverse of :func:`to_independent` (tensors are symmetrised)."""
    def tensor(block):
        t = np.empty((3, 3) + block.shape[1:], dtype=block.dtype)
        for c, (i, j) in enumerate(SYM_PAIRS):
            t[i, j] = block[c]
            t[j, i] = block[c]
        return t
    return BSSNVariables(tensor(u[0:6]), u[6].copy(), tensor(u[7:13]), u[13].copy(),
                         u[14:17].copy(), u[17].copy(), u[18:21].copy())


def map_state(fn, *states):
    return BSSNVariables(*(fn(*leaves) for leaves in zip(*states)))
