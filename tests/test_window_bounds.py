"""Host-side check of the back-projection's table windows (recview_gb300/csrc/rv_bp_ref.cu:
pipe_fill, the int-table window sizes of BpCfg).

The producer warp stages, per view and 64 x 64 tile, the table entries [w0, w0 + nwin) computed
from the tile's four corners; every pixel's index (the truncated detector coordinate
fl(fl(x fcos) + fl(fl(y fsin) + foffset)), the reference's evaluation order) must fall inside,
and nwin must fit the window buffer without the clamp.  The coordinate is monotone in x and in y
under round-to-nearest, so the corners bound it; this test samples random views, tiles and
detector widths up to 8192 pixels with float32 arithmetic and checks both properties.
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32
ALIGN = 4
WIN = ((16 * math.isqrt(63 * 63 * 2 - 1) + 16 + 2 + 3 + ALIGN + 16 + 15) // 16) * 16   # BpCfg, PAD 0


def coord(x, y, c, s, o):
    fy = (f32(y) * s).astype(f32)
    fy = (fy + o).astype(f32)
    return ((f32(x) * c).astype(f32) + fy).astype(f32)


def window(X0, Y0, c, s, o):
    corners = [coord(X0 + cx * 63, Y0 + cy * 63, c, s, o) for cy in (0, 1) for cx in (0, 1)]
    lo, hi = min(corners), max(corners)
    ilo = math.floor(lo) - 2
    lo_a = (ilo & ~(ALIGN - 1)) if ilo >= 0 else -((-ilo + ALIGN - 1) & ~(ALIGN - 1))
    ihi = math.floor(hi) + 3
    return lo_a, ((ihi - lo_a) + 3) & ~3


def test_window_sizes():
    assert WIN == 1472


def test_every_pixel_index_falls_in_its_window():
    rng = np.random.default_rng(17)
    ys, xs = np.meshgrid(np.arange(64), np.arange(64), indexing="ij")
    for _ in range(1500):
        ixdimp = int(rng.choice([64, 512, 2048, 8192]))
        th = rng.uniform(0.0, math.pi)
        c, s = f32(math.cos(th) * 16), f32(-math.sin(th) * 16)
        ixdimh = ixdimp // 2
        fcenter = f32((ixdimh + rng.uniform(-0.25, 0.25) * ixdimp) * 16)
        o = (fcenter - (f32(ixdimh) * (c + s).astype(f32)).astype(f32)).astype(f32)
        tiles = (ixdimp + 63) // 64
        X0, Y0 = 64 * int(rng.integers(tiles)), 64 * int(rng.integers(tiles))
        w0, nwin = window(X0, Y0, c, s, o)
        assert nwin <= WIN                                  # the clamp never binds
        fx = coord(X0 + xs, Y0 + ys, c, s, o)
        v = np.trunc(fx).astype(np.int64)                   # truncation, as the reference's (int)
        assert v.min() >= w0 and v.max() < w0 + nwin
