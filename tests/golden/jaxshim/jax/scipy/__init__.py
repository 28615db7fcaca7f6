"""``jax.scipy`` stand-in (only the sparse iterative solvers are provided)."""
from . import sparse  # noqa: F401
