"""The normalisation's FP32 decision rule, restated in numpy and checked against the reference's
double formula v = (short)(int)(3000 log(I0 / S) + 0.5) (source/general.cpp:2466-2503).

The kernel (recview_gb300/csrc/rv_kernels.cu: norm_fast, norm_exact) decides a sample in FP32
when 3000 L + 0.5 (L = logf of the correctly rounded quotient, carried exactly as p + 0.5 + e)
is farther than its band from an integer n; a flagged sample is then decided by the sign of
I0 - S exp((n - 0.5)/3000) from a float-pair table, and only samples within 1e-9 I0 of the
boundary take FP64.  These tests replay both steps with float32 arithmetic on the inputs
nearest to the rounding boundaries (the float32 I0 closest to each boundary) and require no
wrong decision; two weakened rules must fail on the same inputs, so the inputs do reach the
boundaries.  numpy's float32 log stands in for logf (both within the 1 ulp the band allows 4 of).
"""
from __future__ import annotations

import numpy as np

f32 = np.float32
KMIN, KMAX = -30000, 34000
_N = np.arange(KMIN, KMAX + 1)
_E = np.exp((_N - 0.5) / 3000.0)
E_HI = _E.astype(f32)
E_LO = (_E - E_HI.astype(np.float64)).astype(f32)


def reference(dinc, s):
    return np.trunc(np.log(dinc.astype(np.float64) / s) * 3000.0 + 0.5).astype(np.int64)


def fma32(a, b, c):
    """a*b + c with one rounding (a*b of two float32 is exact in float64)."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def trunc_side(n, positive):
    """Truncation toward zero of a value just above (positive) or below n."""
    return np.where(n > 0, np.where(positive, n, n - 1), np.where(n < 0, np.where(positive, n + 1, n), 0))


def fast_rule(dinc, s, band_scale=f32(12000), band_add=f32(4.3e-4)):
    L = np.log((dinc.astype(np.float64) / s).astype(f32)).astype(f32)
    p = (L * f32(3000)).astype(f32)
    e = fma32(L, np.full_like(L, 3000), -p)
    wh = (p + f32(0.5)).astype(f32)
    N = np.rint(wh).astype(f32)
    t = ((wh - N).astype(f32) + e).astype(f32)
    ulp = (np.abs(L).view(np.int32) & 0x7F800000).view(f32) * f32(2.0 ** -23)
    band = (ulp * band_scale + band_add).astype(f32)
    decided = np.abs(t) > band
    return decided, trunc_side(N.astype(np.int64), t > 0)


def table_rule(dinc, s, split=True):
    L = np.log((dinc.astype(np.float64) / s).astype(f32)).astype(f32)
    n = np.rint((L * f32(3000)).astype(f32) + f32(0.5)).astype(np.int64)
    inside = (n >= KMIN) & (n <= KMAX)
    k = np.clip(n - KMIN, 0, len(_E) - 1)
    sf = s.astype(f32)
    if split:
        ph = (sf * E_HI[k]).astype(f32)
        pl = fma32(sf, E_HI[k], -ph)
        D = (((dinc - ph).astype(f32) - pl).astype(f32) - (sf * E_LO[k]).astype(f32)).astype(f32)
    else:
        D = (dinc - (sf * E_HI[k]).astype(f32)).astype(f32)
    decided = (n == 0) | (inside & (np.abs(D) > (dinc * f32(1e-9)).astype(f32)))
    return decided, trunc_side(n, D > 0)


def near_boundary_samples(rng, m):
    """For random (S, n): the float32 I0 nearest to the boundary S exp((n - 0.5)/3000) and its two
    neighbours, i.e. the hardest inputs the float grid holds (over a million pairs the closest
    land ~1e-10 from the boundary in w)."""
    s = rng.integers(20, 65536, m)
    k = rng.integers(-20000, 30000, m)
    b = (s * np.exp((k - 0.5) / 3000.0)).astype(f32)
    dinc = np.concatenate([np.nextafter(b, f32(0)), b, np.nextafter(b, f32(np.inf))])
    s = np.concatenate([s, s, s])
    ok = np.isfinite(dinc) & (dinc > 0)
    return dinc[ok], s[ok]


def attenuation_samples(rng, m):
    dinc = rng.uniform(15000, 25000, m).astype(f32)
    s = np.maximum(20, dinc * np.exp(-rng.uniform(0, 6, m))).astype(np.int64)
    return dinc, s


def test_fast_rule_never_decides_wrongly():
    rng = np.random.default_rng(11)
    for dinc, s in (near_boundary_samples(rng, 1_000_000), attenuation_samples(rng, 1_000_000)):
        decided, v = fast_rule(dinc, s)
        assert not np.any(decided & (v != reference(dinc, s)))
    dinc, s = attenuation_samples(rng, 1_000_000)
    decided, _ = fast_rule(dinc, s)
    assert np.mean(~decided) < 0.01          # under 1% of ordinary samples reach the recheck


def test_table_rule_never_decides_wrongly():
    rng = np.random.default_rng(12)
    dinc, s = near_boundary_samples(rng, 2_000_000)
    flagged = ~fast_rule(dinc, s)[0]
    dinc, s = dinc[flagged], s[flagged]
    decided, v = table_rule(dinc, s)
    assert not np.any(decided & (v != reference(dinc, s)))
    assert np.mean(decided) > 0.95           # FP64 is left only with samples a hair from the boundary


def test_weakened_rules_fail_on_the_same_inputs():
    rng = np.random.default_rng(13)
    dinc, s = near_boundary_samples(rng, 1_000_000)
    decided, v = fast_rule(dinc, s, band_scale=f32(0), band_add=f32(1e-4))
    assert np.count_nonzero(decided & (v != reference(dinc, s))) > 100
    decided, v = table_rule(dinc, s, split=False)
    assert np.count_nonzero(decided & (v != reference(dinc, s))) > 100
