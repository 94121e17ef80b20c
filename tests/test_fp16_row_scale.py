"""Host-side check of the FP16 row scale (recview_gb300/csrc/rv_kernels.cu: fp16_row_scale).

The FP16 LIN form stores every filtered pair row of a stack under one power-of-two scale chosen
from the filter table alone: a filtered row is the circular convolution of the placed int16 row
(|p| <= 32768) with the kernel h of the filter's even part H[k] = (F[k] + F[-k]) / 2, so
|r| = 100 |q| <= 100 * 32768 * sum|h|, and sum|h| <= sqrt(sum H^2) (Cauchy-Schwarz with
Parseval).  The scale 2^ceil(log2(100 * 32768 * sqrt(sum H^2) / 16384)) then keeps every stored
value below 16384, far from FP16's 65504.  The arithmetic is restated here and checked against
the true kernel norm for every filter kind and size; it runs without a GPU.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from recview_gb300 import abi


def fp16_row_scale(filt: np.ndarray) -> float:
    n = filt.shape[0]
    h = 0.5 * (filt.astype(np.float64) + filt.astype(np.float64)[(n - np.arange(n)) % n])
    bound = 100.0 * 32768.0 * math.sqrt(float((h * h).sum()))
    e = math.ceil(math.log2(bound / 16384.0)) if bound > 0 else 0
    return math.ldexp(1.0, max(-20, min(40, e)))


@pytest.mark.parametrize("kind", [abi.FILT_HAN, abi.FILT_HAM, abi.FILT_RAMP, abi.FILT_PARZN, abi.FILT_BUTER,
                                  abi.FILT_SHEPP])
@pytest.mark.parametrize("ndim", [64, 256, 1024, 4096, 16384])
def test_fp16_scale_bounds_every_row(oracle, kind, ndim):
    filt = oracle.set_filter(kind, ndim)
    n = filt.shape[0]
    H = 0.5 * (filt.astype(np.float64) + filt.astype(np.float64)[(n - np.arange(n)) % n])
    # q = h (*) p with h = (1/n) IDFT(H): the filter pipeline's transform, filter multiply and 1/n
    h = np.fft.ifft(H).real
    l1 = float(np.abs(h).sum())
    assert l1 <= math.sqrt(float((H * H).sum())) * (1 + 1e-9)
    scale = fp16_row_scale(filt)
    worst = 100.0 * 32768.0 * l1 / scale        # largest |r| / scale any int16 row can produce
    assert worst <= 16384.0, (worst, scale)
    # the scale is a power of two (exact scaling) and not needlessly coarse for this filter
    assert math.frexp(scale)[0] == 0.5
    assert worst > 16384.0 / (4 * math.sqrt(n)), (worst, scale)
