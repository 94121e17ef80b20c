"""The filter kernel's transform schedule, restated in numpy float32 and checked bit for bit
against the oracle's radix-2 Stockham FFT (the reference's CFft, source/cfft.cpp:193-369).

The kernel (recview_gb300/csrc/rv_kernels.cu, fft_general_passes and k_filter) regroups the
reference's passes: three general passes per shared-memory round trip over groups of eight
(two per round trip over groups of four for rows below 4096 points), the filter multiply and the
first inverse pass in the same registers as the last forward pass, a swizzled element order in
shared memory, and real parts only after the last inverse pass.  Each regrouping must keep every
butterfly's operands and operation order; this test replays the kernel's index algebra (through
the swizzle) with float32 arithmetic, one rounding per operation as on the GPU, and requires the
oracle's exact bits.  It runs without a GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

F32P = C.POINTER(C.c_float)
f32 = np.float32


def fsw(a):
    return a ^ ((a >> 3) & 14)


class Mem:
    """n complex float32 values stored at swizzled positions, as the kernel's shared buffer."""

    def __init__(self, n):
        self.re = np.zeros(n, f32)
        self.im = np.zeros(n, f32)

    def get(self, idx):
        p = fsw(idx)
        return self.re[p].copy(), self.im[p].copy()

    def put(self, idx, v):
        p = fsw(idx)
        assert len(np.unique(p)) == len(p)
        self.re[p], self.im[p] = v


def cmul(x, w):
    (xr, xi), (wr, wi) = x, w
    return (f32(xr * wr) - f32(xi * wi)).astype(f32), (f32(xr * wi) + f32(xi * wr)).astype(f32)


def cadd(a, b):
    return (a[0] + b[0]).astype(f32), (a[1] + b[1]).astype(f32)


def csub(a, b):
    return (a[0] - b[0]).astype(f32), (a[1] - b[1]).astype(f32)


def pass_table(wr, wi, n):
    """tw[2^l + q] = w[q * (n/2) / 2^l]: pass l's twiddle q, as the library uploads it."""
    half = n // 2
    tr, ti = np.zeros(n, f32), np.zeros(n, f32)
    al = 1
    while al <= half:
        q = np.arange(al)
        tr[al + q], ti[al + q] = wr[q * (half // al)], wi[q * (half // al)]
        al *= 2
    return tr, ti


def general_passes(mem, tr, ti, n):
    """fft_general_passes: triples when n >= 8 x threads (512 threads), else pairs, then singles."""
    half, npw = n // 2, n.bit_length() - 1
    nt = min(half, 512)
    bpt = half // nt
    tw = lambda idx: (tr[idx], ti[idx])  # noqa: E731
    l = 1
    if bpt >= 4:
        eighth = half >> 2
        while l + 2 < npw - 1:
            al, g = 1 << l, np.arange(eighth)
            q = g & (al - 1)
            w1, w2a, w2b = tw(al + q), tw(2 * al + q), tw(3 * al + q)
            P, M = [], []
            for k in range(4):
                x = mem.get(g + k * eighth)
                xb = cmul(mem.get(g + k * eighth + half), w1)
                P.append(cadd(x, xb))
                M.append(csub(x, xb))
            b0, b1, b2, b3 = cmul(P[2], w2a), cmul(M[2], w2b), cmul(P[3], w2a), cmul(M[3], w2b)
            R0, S0, R1, S1 = cadd(P[0], b0), csub(P[0], b0), cadd(M[0], b1), csub(M[0], b1)
            R2, S2, R3, S3 = cadd(P[1], b2), csub(P[1], b2), cadd(M[1], b3), csub(M[1], b3)
            c = [cmul(R2, tw(4 * al + q)), cmul(R3, tw(5 * al + q)), cmul(S2, tw(6 * al + q)), cmul(S3, tw(7 * al + q))]
            lo = [R0, R1, S0, S1]
            out = [cadd(lo[t], c[t]) for t in range(4)] + [csub(lo[t], c[t]) for t in range(4)]
            o = 8 * (g >> l) * al + q
            for t in range(8):
                mem.put(o + t * al, out[t])
            l += 3
    if bpt >= 2:
        quarter = half >> 1
        it = 0
        while l + 1 < npw - 1 and (bpt < 4 or it == 0):
            al, g = 1 << l, np.arange(quarter)
            q = g & (al - 1)
            w = tw(al + q)
            x0, x1 = mem.get(g), cmul(mem.get(g + half), w)
            x2, x3 = mem.get(g + quarter), cmul(mem.get(g + quarter + half), w)
            u0, u1 = cadd(x0, x1), csub(x0, x1)
            v0, v1 = cmul(cadd(x2, x3), tw(2 * al + q)), cmul(csub(x2, x3), tw(3 * al + q))
            o = 4 * (g >> l) * al + q
            mem.put(o, cadd(u0, v0))
            mem.put(o + 2 * al, csub(u0, v0))
            mem.put(o + al, cadd(u1, v1))
            mem.put(o + 3 * al, csub(u1, v1))
            l += 2
            it += 1
    while l < npw - 1:
        al, j = 1 << l, np.arange(half)
        a, b = mem.get(j), cmul(mem.get(j + half), tw(al + (j & (al - 1))))
        o = 2 * j - (j & (al - 1))
        mem.put(o, cadd(a, b))
        mem.put(o + al, csub(a, b))
        l += 1


def kernel_transform(re, im, filt, tr, ti, n):
    """k_filter from the placed row to the real parts after the last inverse pass."""
    half = n // 2
    j = np.arange(half)
    mem = Mem(n)
    # first forward pass (inputs read back to front), stored as adjacent pairs
    a = (re[half - 1 - j], im[half - 1 - j])
    b = (re[n - 1 - j], im[n - 1 - j])
    mem.put(2 * j, cadd(a, b))
    mem.put(2 * j + 1, csub(a, b))
    general_passes(mem, tr, ti, n)
    # last forward pass + filter + first inverse pass in registers
    a = mem.get(j)
    xb = mem.get(j + half)
    cm = cmul(xb, (tr[half + j], ti[half + j]))
    b = (np.where(j == 0, xb[0], cm[0]).astype(f32), np.where(j == 0, xb[1], cm[1]).astype(f32))
    op, om = np.where(j == 0, 0, n - j), np.where(j == 0, half, half - j)
    vp, vm = cadd(a, b), csub(a, b)
    spec = np.zeros(n, f32), np.zeros(n, f32)      # the filtered spectrum, for the oracle's inverse
    yp = ((vp[0] * filt[op]).astype(f32), (vp[1] * filt[op]).astype(f32))
    ym = ((vm[0] * filt[om]).astype(f32), (vm[1] * filt[om]).astype(f32))
    spec[0][op], spec[1][op] = yp
    spec[0][om], spec[1][om] = ym
    k = np.where(j == 0, 0, om)
    lo = (np.where(j == 0, yp[0], ym[0]).astype(f32), np.where(j == 0, yp[1], ym[1]).astype(f32))
    hi = (np.where(j == 0, ym[0], yp[0]).astype(f32), np.where(j == 0, ym[1], yp[1]).astype(f32))
    mem2 = Mem(n)
    mem2.put(2 * k, cadd(lo, hi))
    mem2.put(2 * k + 1, csub(lo, hi))
    general_passes(mem2, tr, ti, n)
    # last inverse pass, real parts only
    ar = mem2.get(j)[0]
    x = mem2.get(j + half)
    brr = (f32(x[0] * tr[half + j]) - f32(x[1] * ti[half + j])).astype(f32)
    out = np.zeros(n, f32)
    out[j], out[j + half] = (ar - brr).astype(f32), (ar + brr).astype(f32)
    return spec, out


@pytest.mark.parametrize("npow", [5, 9, 11, 12, 13, 14])
def test_fused_schedule_matches_oracle_fft(oracle, npow):
    n, half = 1 << npow, 1 << (npow - 1)
    rng = np.random.default_rng(npow)
    wr, wi = np.zeros(half, f32), np.zeros(half, f32)
    oracle.L.rvo_fft_twiddles(npow, wr.ctypes.data_as(F32P), wi.ctypes.data_as(F32P))
    tr, ti = pass_table(wr, wi, n)
    re = rng.normal(0, 1000, n).astype(f32)
    im = np.zeros(n, f32)                        # a placed row is real
    filt = rng.uniform(0, 1, n).astype(f32)
    spec, out = kernel_transform(re, im, filt, tr, ti, n)
    # forward: the oracle's spectrum times the filter, one rounding per component
    fr, fi = oracle.fft(npow, 0, re, im)
    assert np.array_equal((fr * filt).astype(f32).view(np.int32), spec[0].view(np.int32))
    assert np.array_equal((fi * filt).astype(f32).view(np.int32), spec[1].view(np.int32))
    # inverse: the oracle's result is the last pass reversed and scaled by 1/n
    gr, _ = oracle.fft(npow, 1, spec[0], spec[1])
    assert np.array_equal(gr.view(np.int32), (out[::-1] * f32(1.0 / n)).astype(f32).view(np.int32))


def test_swizzle_is_a_permutation_within_16_element_blocks():
    a = np.arange(1 << 16)
    p = fsw(a)
    assert np.array_equal(np.sort(p), a)
    assert np.array_equal(p >> 4, a >> 4)            # stays in its block of 16
    assert np.array_equal(fsw(2 * a[: 1 << 15]) + 1, fsw(2 * a[: 1 << 15] + 1))   # pairs stay adjacent
