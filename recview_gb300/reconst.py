"""Host-side mirror of the reference's reconstruction call: building a RECONST_INFO the way
CGazoDoc::DeconvBackProj / GenerateSinogram fill it (source/gazoDoc.cpp:3929-3951, :3481-3499)
from numpy buffers, and calling the library's C entry points on it.

The sinogram buffer is RecView's: a table of row pointers, row index ``frame * iMultiplex +
slice``, each row ``ixdim`` shorts.  Here the rows live in one contiguous numpy array and the
pointer table is built over it.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


@dataclass
class Dims:
    ixdim: int
    iZooming: int
    iIntpDim: int
    ndimp: int
    ndim: int
    ixdimp: int
    ixdimh: int
    ihoffset: int


def dims(ixdim: int, iInterpolation: int = 2) -> Dims:
    """source/general.cpp:2021-2035 (same integer/log arithmetic)."""
    import math
    iz = iInterpolation - 2 if iInterpolation > 2 else 0
    z = int(math.pow(2.0, iz))
    ndimp = int(math.log(float(ixdim)) / 0.69314718055994530941723212145818) + 1 + iz
    ndim = int(math.pow(2.0, ndimp))
    ixdimp = ixdim * z
    return Dims(ixdim, iz, z, ndimp, ndim, ixdimp, ixdimp // 2, ndim // 2 - 1 - ixdimp // 2)


class ReconInfo:
    """A RECONST_INFO plus the numpy buffers it points into (kept alive by this object)."""

    def __init__(self, rows: np.ndarray, fdeg: np.ndarray, bInc: np.ndarray, *, center: float,
                 fFilter: np.ndarray | None = None, iInterpolation: int = 2, iMultiplex: int = 1,
                 iOffset: int = 0, fexp: np.ndarray | None = None, dReconFlags: int = 0,
                 tilt: float = 0.0, iStartSino: int = 0, iStepSino: int = 1,
                 nviews: int | None = None, maxSinogrLen: int | None = None, iFlag: int = 0,
                 piDrift: np.ndarray | None = None):
        rows = np.ascontiguousarray(rows)
        if rows.ndim == 3:
            rows = rows.reshape(-1, rows.shape[-1])
        assert rows.dtype in (np.int16, np.uint16), rows.dtype
        self.rows = rows
        self.ixdim = rows.shape[1]
        self.d = dims(self.ixdim, iInterpolation)
        self.fdeg = np.ascontiguousarray(fdeg, dtype=np.float32)
        self.bInc = np.ascontiguousarray(bInc, dtype=np.int8)
        self.fexp = np.ascontiguousarray(fexp if fexp is not None else np.arange(len(fdeg)),
                                         dtype=np.float32)
        self.fFilter = None if fFilter is None else np.ascontiguousarray(fFilter, dtype=np.float32)
        self.rowptrs = (C.POINTER(C.c_short) * rows.shape[0])()
        base = rows.ctypes.data
        stride = rows.strides[0]
        for i in range(rows.shape[0]):
            self.rowptrs[i] = C.cast(C.c_void_p(base + i * stride), C.POINTER(C.c_short))
        self.out = np.zeros((self.d.ixdimp, self.d.ixdimp), dtype=np.int32)
        self.nsino = np.zeros(1, dtype=np.int32)
        self.piDrift = None if piDrift is None else np.ascontiguousarray(piDrift, dtype=np.int32)
        ri = abi.RECONST_INFO()
        ri.iStatus = abi.RECONST_INFO_BUSY
        ri.ixdim = self.ixdim
        ri.iInterpolation = iInterpolation
        ri.center = float(center)
        nv = len(self.fdeg) if nviews is None else nviews
        ri.iLenSinogr = nv + 1
        ri.iReconst = _ptr(self.out, C.c_int)
        ri.iStartSino = iStartSino
        ri.iStepSino = iStepSino
        ri.nSinogr = _ptr(self.nsino, C.c_int)
        ri.bInc = C.cast(C.c_void_p(self.bInc.ctypes.data), C.POINTER(C.c_char))
        ri.fdeg = _ptr(self.fdeg, C.c_float)
        ri.fexp = _ptr(self.fexp, C.c_float)
        ri.iMultiplex = iMultiplex
        ri.iOffset = iOffset
        ri.maxSinogrLen = rows.shape[0] if maxSinogrLen is None else maxSinogrLen
        ri.iSinogr = C.cast(self.rowptrs, abi.c_short_pp)
        if self.fFilter is not None:
            ri.fFilter = _ptr(self.fFilter, C.c_float)
        ri.dReconFlags = dReconFlags
        ri.fTiltAngle = tilt
        ri.iFlag = iFlag
        if self.piDrift is not None:
            ri.piDrift = _ptr(self.piDrift, C.c_int)
        self.ri = ri

    @property
    def ref(self):
        return C.byref(self.ri)

    def reset_output(self):
        self.out[...] = 0
        self.nsino[0] = 0
        self.ri.iStatus = abi.RECONST_INFO_BUSY
