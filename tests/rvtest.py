"""Test helpers: ctypes access to the oracle (CPU restatement) and case builders.

The oracle is the checker only; product code never imports this module."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from recview_gb300 import abi, phantom
from recview_gb300.build import build_oracle, REF_LIB
from recview_gb300.reconst import ReconInfo, dims

F32P = C.POINTER(C.c_float)
RIP = C.POINTER(abi.RECONST_INFO)


SP = C.POINTER(C.c_short)
OCT_ARGTYPES = [SP, C.c_longlong, SP, C.c_longlong, C.c_char_p, F32P, C.c_int, C.c_int, C.c_double, C.c_double,
                C.c_int, C.c_int, C.c_int, C.c_int]


def oct_call(fn, rows, ixlen, bInc, fdeg, M, center, dcent, interp, trim, F, iXdim, nof):
    """Runs an offset-CT stitcher with the (oracle / reference) C signature: (rc, rows out)."""
    B = 4 if interp == 0 else (2 if interp == 1 else 1)
    width = iXdim // B
    rows = np.ascontiguousarray(rows, np.int16)
    fdeg = np.ascontiguousarray(fdeg, np.float32)
    out = np.full((max(nof, 1) * M, width), 0x5A5A, np.int16)
    rc = fn(rows.ctypes.data_as(SP), ixlen, out.ctypes.data_as(SP), width, np.asarray(bInc, np.int8).tobytes(),
            fdeg.ctypes.data_as(F32P), len(fdeg), M, center, dcent, interp, trim, F, iXdim)
    return rc, out[:nof * M] if nof > 0 else out[:0]


class Oracle:
    def __init__(self):
        self.L = C.CDLL(str(build_oracle()))
        L = self.L
        L.rvo_set_filter.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, F32P]
        L.rvo_fft_twiddles.argtypes = [C.c_int, F32P, F32P]
        L.rvo_fft_forward.argtypes = [C.c_int, F32P, F32P, F32P, F32P, F32P]
        L.rvo_fft_inverse.argtypes = [C.c_int, F32P, F32P, F32P, F32P, F32P]
        L.rvo_reconstruct.argtypes = [RIP]
        L.rvo_reconstruct_mt.argtypes = [RIP, C.c_int]
        L.rvo_generate_sinogram.argtypes = [RIP]
        L.rvo_reconstruct_lin64.argtypes = [RIP, C.POINTER(C.c_double)]
        L.rvo_reconstruct_lin64_mt.argtypes = [RIP, C.POINTER(C.c_double), C.c_int]
        L.rvo_rescale.argtypes = [C.POINTER(C.c_int), C.c_int, C.c_double, C.c_int, C.c_int,
                                  C.POINTER(C.c_int), C.POINTER(C.c_int)]
        U16P = C.POINTER(C.c_ushort)
        DP = C.POINTER(C.c_double)
        L.rvo_get_axis.argtypes = [U16P, U16P, U16P, C.c_int, C.c_int, C.c_int, DP, DP, DP]
        L.rvo_tv_score.argtypes = [C.POINTER(C.c_int), C.c_int]
        L.rvo_tv_score.restype = C.c_double
        L.rvo_offset_ct_stitch.argtypes = OCT_ARGTYPES
        L.rvo_offset_ct_views.argtypes = [F32P, C.c_int]
        L.rvo_bin_width.argtypes = [C.c_int, C.c_int, C.c_int]
        L.rvo_bin_strip.argtypes = [C.POINTER(C.c_ushort), C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.POINTER(C.c_ushort), C.c_longlong]

    def set_filter(self, kind, ndim, cutoff=0.5, order=2.0):
        t = np.zeros(ndim, np.float32)
        assert self.L.rvo_set_filter(kind, cutoff, order, ndim, t.ctypes.data_as(F32P)) == 0
        return t

    def fft(self, npow, inverse, re, im):
        n = 1 << npow
        tw = np.zeros(n, np.float32)
        self.L.rvo_fft_twiddles(npow, tw.ctypes.data_as(F32P), tw[n // 2:].ctypes.data_as(F32P))
        a = np.ascontiguousarray(re, np.float32).copy()
        b = np.ascontiguousarray(im, np.float32).copy()
        work = np.zeros(4 * n, np.float32)
        f = self.L.rvo_fft_inverse if inverse else self.L.rvo_fft_forward
        f(npow, tw.ctypes.data_as(F32P), tw[n // 2:].ctypes.data_as(F32P), a.ctypes.data_as(F32P),
          b.ctypes.data_as(F32P), work.ctypes.data_as(F32P))
        return a, b

    def reconstruct(self, ri: ReconInfo, threads: int = 1) -> np.ndarray:
        ri.reset_output()
        if threads > 1:
            self.L.rvo_reconstruct_mt(C.byref(ri.ri), threads)
        else:
            self.L.rvo_reconstruct(C.byref(ri.ri))
        return ri.out.copy()

    def generate_sinogram(self, ri: ReconInfo) -> int:
        return self.L.rvo_generate_sinogram(C.byref(ri.ri))

    def lin64(self, ri: ReconInfo, threads: int = 1) -> np.ndarray:
        out = np.zeros((ri.d.ixdimp, ri.d.ixdimp), np.float64)
        if threads > 1:
            self.L.rvo_reconstruct_lin64_mt(C.byref(ri.ri), out.ctypes.data_as(C.POINTER(C.c_double)), threads)
        else:
            self.L.rvo_reconstruct_lin64(C.byref(ri.ri), out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def get_axis(self, s0, s1, flat, offset=0):
        U16P = C.POINTER(C.c_ushort)
        a, b, o = C.c_double(), C.c_double(), C.c_double()
        s0, s1, flat = (np.ascontiguousarray(x, np.uint16) for x in (s0, s1, flat))
        assert self.L.rvo_get_axis(s0.ctypes.data_as(U16P), s1.ctypes.data_as(U16P), flat.ctypes.data_as(U16P),
                                   s0.shape[1], s0.shape[0], offset, C.byref(a), C.byref(b), C.byref(o)) == 0
        return a.value, b.value, o.value

    def tv_score(self, slice_):
        s = np.ascontiguousarray(slice_, np.int32)
        return self.L.rvo_tv_score(s.ctypes.data_as(C.POINTER(C.c_int)), s.shape[0])

    def offset_ct_views(self, fdeg):
        f = np.ascontiguousarray(fdeg, np.float32)
        return self.L.rvo_offset_ct_views(f.ctypes.data_as(F32P), len(f))

    def offset_ct(self, rows, ixlen, bInc, fdeg, M, center, dcent, interp=2, trim=0, F=None, iXdim=None):
        F = F if F is not None else ixlen
        return oct_call(self.L.rvo_offset_ct_stitch, rows, ixlen, bInc, fdeg, M, center, dcent, interp, trim, F,
                        iXdim if iXdim is not None else 2 * F, self.offset_ct_views(fdeg))

    def bin_frames(self, frames: np.ndarray, ixFrm: int, iTrim: int, iInterpolation: int, S: int) -> np.ndarray:
        """Strip assembly of every frame: frames[F, S * bin, ixFrm] uint16 -> [F, S, ixlen]."""
        U16P = C.POINTER(C.c_ushort)
        ixlen = self.L.rvo_bin_width(ixFrm, iTrim, iInterpolation)
        assert ixlen > 0
        frames = np.ascontiguousarray(frames, np.uint16)
        out = np.zeros((frames.shape[0], S, ixlen), np.uint16)
        for f in range(frames.shape[0]):
            rc = self.L.rvo_bin_strip(frames[f].ctypes.data_as(U16P), ixFrm, iTrim, iInterpolation, S,
                                      out[f].ctypes.data_as(U16P), ixlen)
            assert rc == ixlen
        return out

    def rescale(self, slice_, ixdimp, center_user, ipintp=1, ibinning=1):
        s = np.ascontiguousarray(slice_, np.int32).copy()
        imin, imax = C.c_int(), C.c_int()
        self.L.rvo_rescale(s.ctypes.data_as(C.POINTER(C.c_int)), ixdimp, center_user, ipintp, ibinning,
                           C.byref(imin), C.byref(imax))
        return s, imin.value, imax.value


def ref_lib():
    """The reference build (None when the reference checkout was not available)."""
    if not Path(REF_LIB).exists():
        return None
    L = C.CDLL(str(REF_LIB))
    L.rvref_set_filter.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, F32P]
    L.rvref_fbp.argtypes = [RIP]
    L.rvref_gen_sinogram.argtypes = [RIP]
    L.rvref_fft.argtypes = [C.c_int, C.c_int, F32P, F32P]
    U16P = C.POINTER(C.c_ushort)
    L.rvref_get_axis.argtypes = [U16P, U16P, U16P, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double),
                                 C.POINTER(C.c_double)]
    L.rvref_write_tif16.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_char_p, C.c_char_p, C.c_void_p, C.c_int]
    L.rvref_offset_ct.argtypes = OCT_ARGTYPES
    L.rvref_bin_strip.argtypes = [C.POINTER(C.c_short), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.POINTER(C.POINTER(C.c_short))]
    return L


def ref_bin_frames(L, frames: np.ndarray, ixFrm: int, iTrim: int, iInterpolation: int, S: int) -> np.ndarray:
    """The reference build's strip assembly (rvref_bin_strip) of every frame, into rows of the
    width it returns: [F, S * bin, ixFrm] uint16 -> [F, S, ixlen]."""
    B = 4 if iInterpolation == 0 else (2 if iInterpolation == 1 else 1)
    frames = np.ascontiguousarray(frames, np.uint16)
    nf = frames.shape[0]
    rows = np.zeros((nf * S, ixFrm), np.int16)          # wide enough for any width
    ptrs = (C.POINTER(C.c_short) * (nf * S))(*[rows[r].ctypes.data_as(C.POINTER(C.c_short)) for r in range(nf * S)])
    ixlen = None
    for f in range(nf):
        n = L.rvref_bin_strip(frames[f].view(np.int16).ctypes.data_as(C.POINTER(C.c_short)), ixFrm, iTrim, B,
                              0, S, f, ptrs)
        ixlen = n
    return rows[:, :ixlen].reshape(nf, S, ixlen).view(np.uint16).copy()


def fbp_case(seed, W, V, center, interp=2, kind=abi.FILT_SHEPP, cutoff=0.5, flags=0, tilt=0.0,
             skip_every=0, oracle: Oracle | None = None, nviews_span=180.0, **kw) -> ReconInfo:
    """A single-slice reconstruction case: int16 phantom sinogram + RECONST_INFO."""
    sino, fdeg = phantom.sinogram_2d(seed, W, V, center)
    if nviews_span != 180.0:
        fdeg = phantom.angle_table(V, nviews_span)
    d = dims(W, interp)
    F = (oracle or Oracle()).set_filter(kind, d.ndim, cutoff)
    bInc = np.ones(V, np.int8)
    if skip_every:
        bInc[::skip_every] = 0
    return ReconInfo(sino, fdeg, bInc, center=center, fFilter=F, iInterpolation=interp,
                     dReconFlags=flags, tilt=tilt, **kw)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oct_random_case(rng: np.random.Generator, trial: int) -> dict:
    """A random offset-CT stitching case (frames, flags, centre, binning, trim, rows per frame)."""
    F = int(rng.choice([32, 48, 64, 97, 128]))
    interp = int(rng.choice([2, 2, 1, 0, 3]))
    B = 4 if interp == 0 else (2 if interp == 1 else 1)
    T = int(rng.choice([0, 0, 0, 2, 4, 8]))
    M = int(rng.integers(1, 4))
    V = int(rng.choice([40, 60, 61]))
    right = rng.random() < 0.5
    c = F - rng.uniform(2, F / 3) if right else rng.uniform(1, F / 3)
    if rng.random() < 0.3:
        c = float(np.round(c * 4) / 4)          # quarter-pixel centres hit the dc = 0 / 0.5 edges
    dcent = float(rng.choice([0.0, 0.0, rng.uniform(-0.5, 0.5)]))
    ixlen = F // B
    sino, bInc, fdeg = phantom.offset_ct_sinogram(trial, ixlen, V, M, c / B, n_ellipsoids=5)
    if rng.random() < 0.3:
        bInc[rng.integers(2, V, 3)] = 0
    nf = sino.shape[0]
    return dict(rows=np.ascontiguousarray(sino.reshape(nf * M, ixlen)), ixlen=ixlen, bInc=bInc, fdeg=fdeg, M=M,
                center=float(c), dcent=dcent, interp=interp, trim=T, F=F, iXdim=2 * F)
