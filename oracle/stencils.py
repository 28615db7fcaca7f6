"""Finite-difference operators of the reference, restated on NumPy arrays.

Every operator acts along one array axis with periodic wrap-around
(``np.roll`` semantics) and, where a face carries the Sommerfeld code, one-sided
closures on the owned samples ``[start, end)`` of that axis.  Numerators are
accumulated left to right in the reference's term order so that rounding under
cancellation agrees with it.

Sources (uwplasma/JAX_BSSN):
  centred D1 with MAD blend and closures   JAX_BSSN/evolution/derivatives.py:42-163
  upwind D1 (D4/D6 biased, MAD, faces)     JAX_BSSN/evolution/derivatives.py:166-338
  pure D2 with MAD blend and closures      JAX_BSSN/evolution/derivatives.py:341-461
  sixth difference with closures           JAX_BSSN/evolution/derivatives.py:463-599
  boundary data / physical wrappers / KO   JAX_BSSN/evolution/spatial_derivatives.py:18-92
"""

import numpy as np

SOMMERFELD = 1

# Interior stencils as (offset, coefficient) lists in the reference's term order.
UPWIND_D4_FWD = ((-1, -3.0), (0, -10.0), (1, 18.0), (2, -6.0), (3, 1.0))          # /(12 dx)
UPWIND_D4_BWD = ((-3, -1.0), (-2, 6.0), (-1, -18.0), (0, 10.0), (1, 3.0))         # /(12 dx)
UPWIND_D6_FWD = ((-2, 2.0), (-1, -24.0), (0, -35.0), (1, 80.0), (2, -30.0), (3, 8.0), (4, -1.0))  # /(60 dx)
UPWIND_D6_BWD = ((-4, 1.0), (-3, -8.0), (-2, 30.0), (-1, -80.0), (0, 35.0), (1, 24.0), (2, -2.0))  # /(60 dx)
D2_D4 = ((2, -1.0), (1, 16.0), (0, -30.0), (-1, 16.0), (-2, -1.0))                # /(12 dx^2)
D2_D6 = ((3, 1.0 / 90.0), (2, -3.0 / 20.0), (1, 3.0 / 2.0), (0, -49.0 / 18.0),
         (-1, 3.0 / 2.0), (-2, -3.0 / 20.0), (-3, 1.0 / 90.0))                    # /dx^2
D6 = ((3, 1.0), (2, -6.0), (1, 15.0), (0, -20.0), (-1, 15.0), (-2, -6.0), (-3, 1.0))  # /dx^6

# One-sided closures: rows for boundary points 0, 1, ... counted inward from the
# face; columns are the owned samples counted inward from the same face.
D1_LEFT = ((-25.0 / 12.0, 4.0, -3.0, 4.0 / 3.0, -1.0 / 4.0),
           (-1.0 / 4.0, -5.0 / 6.0, 3.0 / 2.0, -1.0 / 2.0, 1.0 / 12.0))
D2_LEFT = ((15.0 / 4.0, -77.0 / 6.0, 107.0 / 6.0, -13.0, 61.0 / 12.0, -5.0 / 6.0),
           (5.0 / 6.0, -5.0 / 4.0, -1.0 / 3.0, 7.0 / 6.0, -1.0 / 2.0, 1.0 / 12.0))
D6_LEFT = ((4.0, -27.0, 78.0, -125.0, 120.0, -69.0, 22.0, -3.0),
           (3.0, -20.0, 57.0, -90.0, 85.0, -48.0, 15.0, -2.0),
           (2.0, -13.0, 36.0, -55.0, 50.0, -27.0, 8.0, -1.0))
# Right closures, written in the reference's order (from the farthest interior
# sample to the face sample); row r serves the point ``end - 1 - r``.
D1_RIGHT = ((1.0 / 4.0, -4.0 / 3.0, 3.0, -4.0, 25.0 / 12.0),
            (-1.0 / 12.0, 1.0 / 2.0, -3.0 / 2.0, 5.0 / 6.0, 1.0 / 4.0))
D2_RIGHT = ((-5.0 / 6.0, 61.0 / 12.0, -13.0, 107.0 / 6.0, -77.0 / 6.0, 15.0 / 4.0),
            (1.0 / 12.0, -1.0 / 2.0, 7.0 / 6.0, -1.0 / 3.0, -5.0 / 4.0, 5.0 / 6.0))
D6_RIGHT = ((-3.0, 22.0, -69.0, 120.0, -125.0, 78.0, -27.0, 4.0),
            (-2.0, 15.0, -48.0, 85.0, -90.0, 57.0, -20.0, 3.0),
            (-1.0, 8.0, -27.0, 50.0, -55.0, 36.0, -13.0, 2.0))


def shifted(f, axis, k):
    """Samples ``f[i + k]`` along ``axis`` with periodic wrap."""
    return np.roll(f, -k, axis=axis)


def ordered_sum(f, axis, table):
    acc = None
    for offset, coefficient in table:
        term = coefficient * shifted(f, axis, offset)
        acc = term if acc is None else acc + term
    return acc


def _apply_closures(derivative, f, axis, start, end, lbc, rbc, left_rows, right_rows, denom):
    if lbc != SOMMERFELD and rbc != SOMMERFELD:
        return derivative
    out = np.moveaxis(derivative, axis, -1).copy()
    src = np.moveaxis(f, axis, -1)
    if lbc == SOMMERFELD:
        for r, row in enumerate(left_rows):
            acc = None
            for c, coefficient in enumerate(row):
                term = coefficient * src[..., start + c]
                acc = term if acc is None else acc + term
            out[..., start + r] = acc / denom
    if rbc == SOMMERFELD:
        width = len(right_rows[0])
        for r, row in enumerate(right_rows):
            acc = None
            for c, coefficient in enumerate(row):
                term = coefficient * src[..., end - width + c]
                acc = term if acc is None else acc + term
            out[..., end - 1 - r] = acc / denom
    return np.moveaxis(out, -1, axis)


def d1(f, axis, dx, lbc=0, rbc=0, q=1.0, start=0, end=None):
    """Centred first derivative: D4, or the MAD blend q*D4+(1-q)*D6 on periodic axes."""
    f = np.asarray(f)
    end = f.shape[axis] if end is None else end
    s = lambda k: shifted(f, axis, k)  # noqa: E731
    d4 = 2 / 3 * (s(1) - s(-1)) / dx + -1 / 12 * (s(2) - s(-2)) / dx
    physical = lbc == SOMMERFELD or rbc == SOMMERFELD
    if q == 1.0 or physical:
        out = d4
    else:
        d6 = (3 / 4 * (s(1) - s(-1)) - 3 / 20 * (s(2) - s(-2)) + 1 / 60 * (s(3) - s(-3))) / dx
        out = q * d4 + (1.0 - q) * d6
    return _apply_closures(out, f, axis, start, end, lbc, rbc, D1_LEFT, D1_RIGHT, dx)


def d2(f, axis, dx, lbc=0, rbc=0, q=1.0, start=0, end=None):
    """Pure second derivative: D4 (5 points) or MAD blend with D6 (7 points)."""
    f = np.asarray(f)
    end = f.shape[axis] if end is None else end
    d4 = ordered_sum(f, axis, D2_D4) / (12.0 * dx ** 2)
    physical = lbc == SOMMERFELD or rbc == SOMMERFELD
    if q == 1.0 or physical:
        out = d4
    else:
        d6 = ordered_sum(f, axis, D2_D6) / dx ** 2
        out = q * d4 + (1.0 - q) * d6
    return _apply_closures(out, f, axis, start, end, lbc, rbc, D2_LEFT, D2_RIGHT, dx ** 2)


def d6(f, axis, dx, lbc=0, rbc=0, start=0, end=None):
    """Undivided-difference sixth derivative [1,-6,15,-20,15,-6,1]/dx^6 with closures."""
    f = np.asarray(f)
    end = f.shape[axis] if end is None else end
    out = ordered_sum(f, axis, D6) / dx ** 6
    return _apply_closures(out, f, axis, start, end, lbc, rbc, D6_LEFT, D6_RIGHT, dx ** 6)


def d1_upwind(f, coefficient, axis, dx, lbc=0, rbc=0, q=1.0, start=0, end=None):
    """Shift-advection derivative selected by the sign of the RHS coefficient.

    Positive coefficient -> forward-biased, negative -> backward-biased, zero ->
    centred.  A Sommerfeld face forces D4 on the axis and replaces the three
    outer owned samples at that face by the closed centred D4 derivative.
    """
    f = np.asarray(f)
    end = f.shape[axis] if end is None else end
    s = lambda k: shifted(f, axis, k)  # noqa: E731
    fwd = ordered_sum(f, axis, UPWIND_D4_FWD) / (12.0 * dx)
    bwd = ordered_sum(f, axis, UPWIND_D4_BWD) / (12.0 * dx)
    ctr = (2.0 / 3.0 * (s(1) - s(-1)) - 1.0 / 12.0 * (s(2) - s(-2))) / dx
    physical = lbc == SOMMERFELD or rbc == SOMMERFELD
    if not (q == 1.0 or physical):
        fwd6 = ordered_sum(f, axis, UPWIND_D6_FWD) / (60.0 * dx)
        bwd6 = ordered_sum(f, axis, UPWIND_D6_BWD) / (60.0 * dx)
        ctr6 = (3.0 / 4.0 * (s(1) - s(-1)) - 3.0 / 20.0 * (s(2) - s(-2))
                + 1.0 / 60.0 * (s(3) - s(-3))) / dx
        fwd = q * fwd + (1.0 - q) * fwd6
        bwd = q * bwd + (1.0 - q) * bwd6
        ctr = q * ctr + (1.0 - q) * ctr6
    c = np.asarray(coefficient)
    out = np.where(c > 0.0, fwd, np.where(c < 0.0, bwd, ctr))
    if not physical:
        return out
    centred = d1(f, axis, dx, lbc, rbc, 1.0, start, end)
    width = min(3, f.shape[axis])
    sel = np.moveaxis(out, axis, -1).copy()
    cen = np.moveaxis(centred, axis, -1)
    n = sel.shape[-1]
    if lbc == SOMMERFELD:
        lo = min(max(start, 0), n - width)
        sel[..., lo:lo + width] = cen[..., lo:lo + width]
    if rbc == SOMMERFELD:
        lo = min(max(end - width, 0), n - width)
        sel[..., lo:lo + width] = cen[..., lo:lo + width]
    return np.moveaxis(sel, -1, axis)


# --- parameter-aware wrappers (JAX_BSSN/evolution/spatial_derivatives.py:18-92) ---

def axis_data(shape, d, params):
    """Face codes, owned range, MAD weight and reduced flag for direction d."""
    codes = (params.xl_bc, params.xr_bc, params.yl_bc, params.yr_bc, params.zl_bc, params.zr_bc)
    lbc, rbc = int(codes[2 * d]), int(codes[2 * d + 1])
    q = 1.0 if (lbc == SOMMERFELD or rbc == SOMMERFELD) else float(params.mad_q)
    lbc = lbc if params.owned_faces[2 * d] else 0
    rbc = rbc if params.owned_faces[2 * d + 1] else 0
    start = int(params.guard_cells)
    count = shape[len(shape) - 3 + d] if params.owned_shape is None else params.owned_shape[d]
    if params.reduced_axes is not None:
        reduced = bool(params.reduced_axes[d])
    elif params.owned_shape is not None:
        reduced = count == 1
    else:
        reduced = False
    return lbc, rbc, start, start + int(count), q, reduced


def D1(f, d, params):
    f = np.asarray(f)
    lbc, rbc, start, end, q, reduced = axis_data(f.shape, d, params)
    if reduced:
        return np.zeros_like(f)
    return d1(f, f.ndim - 3 + d, params.dx, lbc, rbc, q, start, end)


def D2(f, d, params):
    f = np.asarray(f)
    lbc, rbc, start, end, q, reduced = axis_data(f.shape, d, params)
    if reduced:
        return np.zeros_like(f)
    return d2(f, f.ndim - 3 + d, params.dx, lbc, rbc, q, start, end)


def D1_upwind(f, coefficient, d, params):
    f = np.asarray(f)
    lbc, rbc, start, end, q, reduced = axis_data(f.shape, d, params)
    if reduced:
        return np.zeros_like(f)
    return d1_upwind(f, coefficient, f.ndim - 3 + d, params.dx, lbc, rbc, q, start, end)


def kreiss_oliger(f, params):
    """nu/64 * sum_d h^5 D6_d f (JAX_BSSN/evolution/spatial_derivatives.py:81-92)."""
    f = np.asarray(f)
    h = params.dx
    total = 0
    for d in range(3):
        lbc, rbc, start, end, _, reduced = axis_data(f.shape, d, params)
        if reduced:
            term = np.zeros_like(f)
        else:
            term = h ** 5 * d6(f, f.ndim - 3 + d, h, lbc, rbc, start, end)
        total = total + term
    return params.nu / 64 * total


def mixed(f, inner, outer, params, first=None):
    """Second derivative d_outer d_inner f: D2 when equal, else D1(D1(f, inner), outer)."""
    if inner == outer:
        return D2(f, outer, params)
    base = D1(f, inner, params) if first is None else first
    return D1(base, outer, params)
