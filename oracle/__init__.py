"""CPU float64 oracle for the JAX_BSSN evolution hot path.

TEST INFRASTRUCTURE ONLY.  This package is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it.
The product path (``jax_bssn_gb300``) never calls into it and fails loudly when
its CUDA library is missing.

It restates, in NumPy, the reference's algorithm for the path
(uwplasma/JAX_BSSN): finite-difference stencils with their boundary closures,
the BSSN right-hand side in the W formulation, the algebraic projection, RK4,
Sommerfeld faces, constraints, FMR prolongation/injection and the Cartoon
reconstructions.  Each function cites the reference file:line it follows.
Evaluation order inside each stencil numerator follows the reference so that
rounding agrees where cancellation amplifies it.

Parity of this oracle is pinned against golden vectors produced by running
the unmodified reference source under a NumPy ``jax`` stand-in
(``tests/golden/make_golden.py``; fixtures in ``tests/golden/*.npz``).
"""

from .state import BSSNParameters, BSSNVariables, pack_state, unpack_state  # noqa: F401
