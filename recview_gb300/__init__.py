"""recview_gb300 -- GB300-native convolution back-projection behind RecView's C entry points.

The product is the shared library ``librecview_gb300.so`` (CUDA kernels for sm_103a + the C ABI
declared in ``include/recview_gb300.h``).  This package loads it with ctypes and offers thin
Python helpers over the same entry points.  There is no CPU fallback: every helper calls the
library, and loading fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import abi
from .reconst import ReconInfo, dims

__all__ = ["lib", "ReconInfo", "dims", "Stack", "set_filter", "reconstruct_slice", "normalise",
           "last_error", "LibraryNotBuilt"]

_PKG = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("RECVIEW_GB300_LIB", _PKG / "librecview_gb300.so"))
_lib: C.CDLL | None = None


class LibraryNotBuilt(RuntimeError):
    pass


def lib() -> C.CDLL:
    """The bound C library (raises LibraryNotBuilt if the .so is missing)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise LibraryNotBuilt(f"{LIB_PATH} not found: run `python -m recview_gb300.build` "
                                  "(or __graft_entry__.build()) first")
        _lib = abi.bind(C.CDLL(str(LIB_PATH)))
    return _lib


def last_error() -> tuple[int, str]:
    L = lib()
    return L.RvGetLastError(), (L.RvGetLastErrorMessage() or b"").decode()


def set_filter(kind: int, ndim: int, cutoff: float = 0.5, order: float = 2.0) -> np.ndarray:
    """Filter table in RecView's one-sided layout (CGazoDoc::SetFilter)."""
    out = np.zeros(ndim, dtype=np.float32)
    rc = lib().RvSetFilter(kind, cutoff, order, ndim, out.ctypes.data_as(C.POINTER(C.c_float)))
    if rc:
        raise ValueError(f"RvSetFilter failed: {rc}")
    return out


def reconstruct_slice(ri: ReconInfo, idev: int = 0, report: bool = False, streams: bool = False) -> np.ndarray:
    """CudaReconstHost on a ReconInfo; returns the int32 slice (also left in ri.out)."""
    lib().CudaReconstHost(ri.ref, idev, report, streams)
    if ri.ri.iStatus == abi.RECONST_INFO_ERROR:
        code, msg = last_error()
        raise RuntimeError(f"CudaReconstHost failed ({code}): {msg}")
    return ri.out


def normalise(ri: ReconInfo, idev: int = 0) -> None:
    """CudaSinogramHost: flat/dark log normalisation of ri.rows in place."""
    lib().CudaSinogramHost(ri.ref, idev, False)
    if ri.ri.iStatus == abi.RECONST_INFO_ERROR:
        code, msg = last_error()
        raise RuntimeError(f"CudaSinogramHost failed ({code}): {msg}")


class Stack:
    """RvStack: raw uint16 frames of many detector rows -> slices, on the device."""

    def __init__(self, *, ixdim: int, nframes: int, nslices: int, center: float, bInc, fdeg, fexp,
                 fFilter, iInterpolation: int = 2, tilt: float = 0.0, mode: int = abi.MODE_REF,
                 flags: int = 0, iFlag: int = 0, input_is_sinogram: bool = False, iTrim: int = 0,
                 raw_width: int = 0):
        self._keep = [np.ascontiguousarray(bInc, dtype=np.int8), np.ascontiguousarray(fdeg, dtype=np.float32),
                      np.ascontiguousarray(fexp, dtype=np.float32), np.ascontiguousarray(fFilter, dtype=np.float32)]
        b, fd, fe, ff = self._keep
        desc = abi.RvStackDesc()
        desc.ixdim = ixdim
        desc.iInterpolation = iInterpolation
        desc.center = center
        desc.nframes = nframes
        desc.nslices = nslices
        desc.bInc = C.cast(C.c_void_p(b.ctypes.data), C.POINTER(C.c_char))
        desc.fdeg = fd.ctypes.data_as(C.POINTER(C.c_float))
        desc.fexp = fe.ctypes.data_as(C.POINTER(C.c_float))
        desc.fTiltAngle = tilt
        desc.fFilter = ff.ctypes.data_as(C.POINTER(C.c_float))
        desc.dReconFlags = flags
        desc.iFlag = iFlag
        desc.mode = mode
        desc.input_is_sinogram = 1 if input_is_sinogram else 0
        desc.iTrim = iTrim
        desc.iRawWidth = raw_width
        h = C.c_void_p()
        rc = lib().RvStackCreate(C.byref(desc), C.byref(h))
        if rc:
            raise RuntimeError(f"RvStackCreate failed ({rc}): {last_error()[1]}")
        self.h = h
        self.mode = mode
        self.nslices = nslices
        self.ixdimp = lib().RvStackOutputDim(h)
        self.nviews = lib().RvStackNumViews(h)

    @property
    def out_dtype(self):
        return np.int32 if self.mode == abi.MODE_REF else np.float32

    def run_host(self, raw: np.ndarray, out: np.ndarray | None = None, stream: int = 0) -> np.ndarray:
        raw = np.ascontiguousarray(raw)
        if out is None:
            out = np.empty((self.nslices, self.ixdimp, self.ixdimp), dtype=self.out_dtype)
        rc = lib().RvStackRunHost(self.h, C.c_void_p(raw.ctypes.data), C.c_void_p(out.ctypes.data), C.c_void_p(stream))
        if rc:
            raise RuntimeError(f"RvStackRunHost failed ({rc}): {last_error()[1]}")
        return out

    def run_device(self, d_raw: int, d_out: int, stream: int = 0) -> None:
        rc = lib().RvStackRunDevice(self.h, C.c_void_p(d_raw), C.c_void_p(d_out), C.c_void_p(stream))
        if rc:
            raise RuntimeError(f"RvStackRunDevice failed ({rc}): {last_error()[1]}")

    def timings(self) -> tuple[float, float, float]:
        t = (C.c_float * 3)()
        lib().RvStackLastTimings(self.h, t)
        return t[0], t[1], t[2]

    def launches(self) -> int:
        return lib().RvStackLastLaunchCount(self.h)

    def close(self):
        if getattr(self, "h", None):
            lib().RvStackDestroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
