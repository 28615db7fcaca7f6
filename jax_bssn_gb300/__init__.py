"""GB300-native (sm_103a) kernels for the JAX_BSSN evolution hot path.

Mirrors the reference package layout for the hot path: ``bssn`` (state
contract), ``evolution`` (RHS, projection, RK4).  All arithmetic runs in the
in-tree CUDA library ``lib/libbssn_gb300.so``; there is no CPU fallback.
"""

__version__ = "0.1.0"

from ._device import arithmetic, current_arithmetic, set_arithmetic  # noqa: E402,F401
from .bssn.variables import BSSNParameters, BSSNVariables  # noqa: E402,F401
