"""Host-side check of the back-projection's ray-aligned lane footprints (recview_gb300/csrc/
rv_bp_ref.cu: ray_shift, ray_coords, the accumulator exchange in bp_ref_tile_ws).

For every regime (orientation and shear k in [-NQ, NQ]) the CW consumer warps' 64 / CW x 2
register slots per lane must cover the 64 x 64 tile exactly once, and the exchange that moves
the accumulators when a chunk of views changes regime must hand every new slot the old slot of
the same pixel.  The kernels' parity tests only reach the regimes their view sets visit; this
test walks all pairs.  The index arithmetic is restated from the kernel; it runs without a GPU.
"""
from __future__ import annotations

import numpy as np
import pytest


def ray_shift(j, regime, nq):
    k = (regime >> 1) - nq
    return (2 * j * k + nq + 128 * nq) // (2 * nq) - 64     # the numerator is positive: C's / is floor


def layout(regime, cw, nq):
    """Pixel (x, y) and exchange slot of every (warp, lane, q, p) under a regime."""
    q_n = 64 // cw
    w, j, q, p = np.meshgrid(np.arange(cw), np.arange(32), np.arange(q_n), np.arange(2), indexing="ij")
    u = (w + ray_shift(j, regime, nq) + cw * q) & 63
    f = j + 32 * p
    x, y = (f, u) if regime & 1 else (u, f)
    slot = (2 * q + p) * (32 * cw) + w * 32 + j
    return w, j, q, p, x, y, slot


@pytest.mark.parametrize("cw,nq", [(8, 12), (16, 8)])
def test_every_regime_covers_the_tile_once(cw, nq):
    for regime in [o | ((k + nq) << 1) for o in (0, 1) for k in range(-nq, nq + 1)]:
        *_, x, y, _ = layout(regime, cw, nq)
        cover = np.zeros((64, 64), np.int64)
        np.add.at(cover, (y.ravel(), x.ravel()), 1)
        assert np.all(cover == 1), regime


@pytest.mark.parametrize("cw,nq", [(8, 12), (16, 8)])
def test_exchange_hands_each_pixel_its_old_slot(cw, nq):
    regimes = [o | ((k + nq) << 1) for o in (0, 1) for k in range(-nq, nq + 1)]
    nc = 32 * cw
    for ro in regimes:
        *_, xo, yo, so = layout(ro, cw, nq)
        owner = np.full((64, 64), -1, np.int64)
        owner[yo.ravel(), xo.ravel()] = so.ravel()
        oo = ro & 1
        for rn in regimes:
            w, j, q, p, xn, yn, _ = layout(rn, cw, nq)
            # the kernel's source index for new slot (q, p) of thread (w, j)
            a = xn if oo else yn
            c = yn if oo else xn
            jj, pp = a & 31, a >> 5
            m = (c - ray_shift(jj, ro, nq)) & 63
            src = ((m // cw) * 2 + pp) * nc + (m % cw) * 32 + jj
            assert src.min() >= 0 and src.max() < 4096
            assert np.array_equal(src, owner[yn, xn]), (ro, rn)
