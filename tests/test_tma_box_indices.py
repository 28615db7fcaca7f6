"""Shared-memory indices of the FP32 TMA box kernels near Sommerfeld faces,
replayed on the CPU.

The box kernels (jax_bssn_gb300/csrc/bssn_rhs.cu: box_origin, row_code,
BoxRing::start, d1_row / d2_row / ko_row and the interior stencils) read every
tap of every thread -- valid or not -- from a shared-memory box whose origin
is lowered in tiles that hold the rows next to an upper Sommerfeld face.
This test restates those rules and checks, for every tile and thread of
several grid shapes (the upper-face rows at every position within a tile),
that each tap lies inside its box and that every valid sample's taps lie
inside the padded block.  Samples outside the launch box read as if at the
tile origin with interior stencils; without that rule the lowered boxes end
below the tile's samples beyond the face.
"""

import itertools

import pytest

AZ, AY, AX, AHZ = 32, 4, 4, 40
# kind: (box extent y, box extent x, reach below an upper face)
KINDS = {"V2": (AY + 4, AX + 4, 5), "DX": (AY + 4, AX, 4), "DY": (AY, AX, 4), "V3": (AY + 6, AX + 6, 7)}
# stencils each box kind serves along (x, y, z)
OPS = {"V2": (("D2", "D1"), ("D2", "D1"), ("D2", "D1")), "DX": ((), ("D1",), ("D1",)), "DY": ((), (), ("D1",)),
       "V3": (("T",), ("T",), ("T",))}


def _upper_face_in(start, end, t0, extent, blo, bhi):
    xf = end - 1
    lo, hi = max(t0, xf - 2, blo), min(t0 + extent - 1, xf - 1, bhi - 1)
    return xf if lo <= hi else None


def _origin(kind, tile, axes, box):
    hy_box, hx_box, reach = KINDS[kind]
    hx, hy = (hx_box - AX) // 2, (hy_box - AY) // 2
    x0, y0, z0 = tile
    ox, oy, oz = -hx, -hy, -4
    f = _upper_face_in(*axes[0], x0, AX, *box[0]) if hx else None
    if f is not None:
        ox = min(ox, f - reach - x0)
    f = _upper_face_in(*axes[1], y0, AY, *box[1]) if hy else None
    if f is not None:
        oy = min(oy, f - reach - y0)
    f = _upper_face_in(*axes[2], z0, AZ, *box[2])
    if f is not None and f - reach - z0 < oz:
        oz = -((z0 - (f - reach) + 3) & ~3)
    return ox, oy, oz


def _row_code(start, end, c):
    r = end - 1 - c
    if r in (1, 2):
        return -r
    r = c - start
    return r if r in (1, 2) else 0


def _taps(op, code):
    """Offsets an operator reads along its axis at a row code: the centred
    taps always (every sample reads them first), and on the one-sided rows the
    outer taps beyond them."""
    side = 1 if code > 0 else -1
    if op == "D1":
        return [-2, -1, 1, 2] + ([0, 3 * side] if abs(code) == 1 else [])
    if op == "D2":
        return [-2, -1, 0, 1, 2] + ([3 * side, 4 * side] if abs(code) == 1 else [])
    window = list(range(-3, 4))       # transport: the centred 7-tap window
    if code == 0:
        return window
    return window + [side * o for o in ((4, 5, 6) if abs(code) == 1 else (4, 5))]


def _out_of_box_taps(n, ghost=4):
    padded = [m + 2 * ghost for m in n]
    axes = [(ghost, ghost + m) for m in n]            # owned [start, end)
    box = [(s + 1, e - 1) for s, e in axes]           # without the face planes
    z_base = box[2][0] & ~3
    tiles = [range(box[0][0], box[0][1], AX), range(box[1][0], box[1][1], AY), range(z_base, box[2][1], AZ)]
    bad = 0
    for tile in itertools.product(*tiles):
        origins = {k: _origin(k, tile, axes, box) for k in KINDS}
        for off in itertools.product(range(AX), range(AY), range(AZ)):
            pos = [t + o for t, o in zip(tile, off)]
            valid = all(lo <= c < hi for c, (lo, hi) in zip(pos, box))
            local = off if valid else (0, 0, 0)
            codes = [_row_code(*axes[d], pos[d]) for d in range(3)] if valid else [0, 0, 0]
            for kind, (hy_box, hx_box, _) in KINDS.items():
                o = origins[kind]
                assert (tile[2] + o[2]) % 4 == 0          # 16-byte box origin in z
                centre = [local[d] - o[d] for d in range(3)]
                for d, ops in enumerate(OPS[kind]):
                    for op in ops:
                        for t in _taps(op, codes[d]):
                            ix = list(centre)
                            ix[d] += t
                            if not (0 <= ix[0] < hx_box and 0 <= ix[1] < hy_box and 0 <= ix[2] < AHZ):
                                bad += 1
                            elif valid:
                                g = [tile[i] + o[i] + ix[i] for i in range(3)]
                                assert all(0 <= g[i] < padded[i] for i in range(3))
    return bad


@pytest.mark.parametrize("shape", [(24, 20, 24), (23, 22, 20), (26, 21, 28), (18, 25, 24), (17, 19, 20)])
def test_box_taps_stay_in_their_boxes(shape):
    assert _out_of_box_taps(shape) == 0


# ---------------------------------------------------------------------------
# The first-derivative kernel (k_first_derivs_tma<true>): 32 (z) x 8 (y) x 4
# (x) tiles, four z samples per thread, 40 x 12 x 8 boxes (halo 4 in z, 2 in y
# and x) over the whole box, face planes included, with the D1 closure rows
# (d1_code, d1_origin, the z window of twelve samples and the ld4 taps).
TZ, TY, TX = 32, 8, 4
DHZ, DHY, DHX = TZ + 8, TY + 4, TX + 4


def _d1_code(start, end, c, closed=True):
    if not closed:
        return 0
    r = end - 1 - c
    if r in (0, 1):
        return -(r + 1)
    r = c - start
    return r + 1 if r in (0, 1) else 0


def _d1_origin(start, end, t0, extent, blo, bhi, closed=True):
    if not closed:
        return -2
    xf = end - 1
    lo, hi = max(t0, xf - 1, blo), min(t0 + extent - 1, xf, bhi - 1)
    return min(-2, xf - 4 - t0) if lo <= hi else -2


def _derivative_taps_out_of_box(n, periodic_y=False, ghost=4):
    padded = [m + 2 * ghost for m in n]
    axes = [(ghost, ghost + m) for m in n]
    closed = [True, not periodic_y, True]
    # the launch box: the owned samples, grown by the composition reach (2) on
    # a periodic axis
    box = [(s - (0 if c else 2), e + (0 if c else 2)) for (s, e), c in zip(axes, closed)]
    z_base = box[2][0] & ~3
    bad = 0
    for x0, y0, z0 in itertools.product(range(box[0][0], box[0][1], TX), range(box[1][0], box[1][1], TY),
                                        range(z_base, box[2][1], TZ)):
        assert (z0 - 4) % 4 == 0
        ox = _d1_origin(*axes[0], x0, TX, *box[0], closed[0])
        oy = _d1_origin(*axes[1], y0, TY, *box[1], closed[1])
        for tx, ty, tz4 in itertools.product(range(TX), range(TY), range(TZ // 4)):
            x, y, zq = x0 + tx, y0 + ty, z0 + 4 * tz4
            col = box[0][0] <= x < box[0][1] and box[1][0] <= y < box[1][1]
            rx, ry = (tx, ty) if col else (0, 0)
            base = ((rx - ox) * DHY + (ry - oy)) * DHZ + 4 + 4 * tz4
            cx = _d1_code(*axes[0], x, closed[0]) if col else 0
            cy = _d1_code(*axes[1], y, closed[1]) if col else 0
            reads = [base - 4 + i for i in range(12)]           # the z window
            for c, st in ((cx, DHY * DHZ), (cy, DHZ)):
                if c:
                    sg = st if c > 0 else -st
                    offs = [0, sg, 2 * sg, 3 * sg, 4 * sg if abs(c) == 1 else -sg]
                else:
                    offs = [-2 * st, -st, st, 2 * st]
                reads += [base + o + i for o in offs for i in range(4)]
            for r in reads:
                if not 0 <= r < DHZ * DHY * DHX:
                    bad += 1
                    continue
                if col:   # a valid column reads real samples of the padded block
                    g = (x0 + ox + r // (DHY * DHZ), y0 + oy + (r // DHZ) % DHY, z0 - 4 + r % DHZ)
                    zs = [zq + j for j in range(4) if box[2][0] <= zq + j < box[2][1]]
                    if zs and (r % DHZ) in range(4 + 4 * tz4 - 4, 4 + 4 * tz4 + 8):
                        bad += not (0 <= g[0] < padded[0] and 0 <= g[1] < padded[1])
            # the z closure taps of every sample stay inside the window
            for j in range(4):
                cz = _d1_code(*axes[2], zq + j, closed[2]) if col else 0
                if cz:
                    up = cz < 0
                    idx = [4 + j + (-k if up else k) for k in (1, 2, 3)]
                    idx.append(4 + j + ((-4 if up else 4) if abs(cz) == 1 else (1 if up else -1)))
                    assert all(0 <= i < 12 for i in idx)
    return bad


# the upper faces at every position within a tile along x (4) and y (8)
D1_SHAPES = [((16 + k, 17 + k, 20 + k), False) for k in range(8)] + [((21, 23, 24), True), ((128, 128, 128), False)]


@pytest.mark.parametrize("shape,periodic_y", D1_SHAPES)
def test_first_derivative_taps_stay_in_their_boxes(shape, periodic_y):
    assert _derivative_taps_out_of_box(shape, periodic_y) == 0


def test_first_derivative_replay_finds_unlowered_boxes(monkeypatch):
    """The replay is sensitive: boxes left at halo 2 in tiles that hold an
    upper face plane read below their boxes."""
    import sys
    monkeypatch.setattr(sys.modules[__name__], "_d1_origin", lambda *a, **k: -2)
    assert sum(_derivative_taps_out_of_box(shape, py) for shape, py in D1_SHAPES[:8]) > 0
