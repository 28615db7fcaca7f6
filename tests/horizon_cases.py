"""Analytic Schwarzschild slices for the apparent-horizon tests.

The reference suite's fixtures (tests/test_apparent_horizon.py:24-70): the
physical Schwarzschild metric and extrinsic curvature in isotropic or
Kerr-Schild slicing, pulled back to stretched and shifted coordinates so the
horizon becomes a coordinate ellipsoid of semi-axes mass / (2 scale), stored
as a radial line, a signed x-z plane or a Cartesian volume.
"""

import numpy as np

MASS = 2.0


def schwarzschild_tensors(position, mass=MASS, slicing="isotropic", scale=(1.0, 1.0, 1.0),
                          center=(0.0, 0.0, 0.0)):
    stretched = [factor * (q - shift) for q, factor, shift in zip(position, scale, center)]
    radius = np.sqrt(sum(q ** 2 for q in stretched))
    identity = np.eye(3).reshape((3, 3) + (1,) * radius.ndim)
    if slicing == "isotropic":
        gamma = identity * (1 + mass / (2 * radius)) ** 4
        kij = np.zeros_like(gamma)
    else:
        normal = np.stack([q / radius for q in stretched])
        outer = normal[:, None] * normal[None, :]
        gamma = identity + (2 * mass / radius) * outer
        kij = (2 * mass / (radius ** 2 * np.sqrt(1 + 2 * mass / radius))) * (identity - (2 + mass / radius) * outer)
    factors = np.asarray(scale)
    pullback = (factors[:, None] * factors[None, :]).reshape((3, 3) + (1,) * radius.ndim)
    return gamma * pullback, kij * pullback


def schwarzschild_line(dx=0.02, extent=8.0, **keywords):
    radius = (np.arange(int(round(extent / dx))) + 0.5) * dx
    zero = np.zeros_like(radius)
    return (radius,) + schwarzschild_tensors((radius, zero, zero), **keywords)


def schwarzschild_plane(dx=0.05, extent=4.0, stretch=1.0, center_z=0.0, **keywords):
    count = 2 * int(round(extent / dx))
    axis = (np.arange(count) - (count - 1) / 2) * dx
    first, second = np.meshgrid(axis, axis, indexing="ij")
    tensors = schwarzschild_tensors((first, np.zeros_like(first), second), scale=(1.0, 1.0, stretch),
                                    center=(0.0, 0.0, center_z), **keywords)
    return (axis, axis) + tensors


def schwarzschild_volume(dx=0.0625, extent=2.5, **keywords):
    count = 2 * int(round(extent / dx))
    axis = (np.arange(count) - (count - 1) / 2) * dx
    return (axis, axis, axis) + schwarzschild_tensors(np.meshgrid(axis, axis, axis, indexing="ij"), **keywords)


def layout_case(layout, slicing, volume_dx=0.05, volume_extent=3.0):
    """(axes, gamma, Kij, mass, exact coordinate radius) of one exact-mass case."""
    mass = 1.0 if slicing == "kerr_schild" else MASS
    options = dict(mass=mass, slicing=slicing)
    if layout == "line":
        r, gamma, kij = schwarzschild_line(**options)
        axes = (r,)
    elif layout == "plane":
        x, z, gamma, kij = schwarzschild_plane(**options)
        axes = (x, z)
    else:
        x, y, z, gamma, kij = schwarzschild_volume(dx=volume_dx, extent=volume_extent, **options)
        axes = (x, y, z)
    exact = 2 * mass if slicing == "kerr_schild" else mass / 2
    return axes, gamma, kij, mass, exact
