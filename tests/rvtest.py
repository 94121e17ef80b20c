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
        L.rvo_rescale.argtypes = [C.POINTER(C.c_int), C.c_int, C.c_double, C.c_int, C.c_int,
                                  C.POINTER(C.c_int), C.POINTER(C.c_int)]
        U16P = C.POINTER(C.c_ushort)
        DP = C.POINTER(C.c_double)
        L.rvo_get_axis.argtypes = [U16P, U16P, U16P, C.c_int, C.c_int, C.c_int, DP, DP, DP]
        L.rvo_tv_score.argtypes = [C.POINTER(C.c_int), C.c_int]
        L.rvo_tv_score.restype = C.c_double

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

    def lin64(self, ri: ReconInfo) -> np.ndarray:
        out = np.zeros((ri.d.ixdimp, ri.d.ixdimp), np.float64)
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
    return L


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
