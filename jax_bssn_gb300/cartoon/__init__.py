"""Cartoon symmetry reductions on GB300 (mirrors JAX_BSSN.cartoon).

``axisymmetry``: compact (Nrho+4, 1, Nz) states about the z axis;
``spherical_symmetry``: compact (Nr+4, 1, 1) radial states.  Reconstruction,
RHS, RK4 and constraints run in ``libbssn_gb300.so``.
"""
