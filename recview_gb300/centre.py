"""Centre search helpers over the C ABI: synthetic scans, GetAxis, the learned and plain searches,
and network training (all the work runs in the library's kernels; this module is plumbing).

The plain method is the axis-scan sweep (source/gazoDoc.cpp:1994-2024) of 2*40+1 trial centres
0.5 px apart around GetAxis's estimate (source/gazoDoc.cpp:4036-4626), scored by the library's
sharpness criterion on trial slices reconstructed with a Hann filter of cutoff 0.25.  The learned
search (RvCentreSearch with a network) reconstructs only the trials around the network's proposal.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import abi, lib, last_error, set_filter, dims

FP = C.POINTER(C.c_float)


def _fp(a: np.ndarray):
    return a.ctypes.data_as(FP)


@dataclass
class Scan:
    raw: object          # torch uint16-as-int16 [(frames+1), S, W] on the device
    sino: object         # torch int16 normalised rows, same shape
    bInc: np.ndarray
    fdeg: np.ndarray
    centre: float        # true centre (ri->center convention)


def make_scan(seed: int, offset: float, W: int = 2048, views: int = 1800, S: int = 4, n_ellipsoids: int = 40) -> Scan:
    """Raw frames (flat, `views` samples over 180 degrees, flat, dark) and their normalised rows."""
    import torch
    L = lib()
    deg = (np.arange(views) * (180.0 / views)).astype(np.float32)
    dev = torch.device("cuda")
    raw = torch.empty((views + 3, S, W), dtype=torch.int16, device=dev)
    binc = np.zeros(views + 2, np.int8)
    fdeg = np.zeros(views + 2, np.float32)
    fexp = np.zeros(views + 2, np.float32)
    centre = (W - 1) / 2.0 + offset
    rc = L.RvPhantomFrames(seed, W, S, _fp(deg), views, centre, n_ellipsoids, C.c_void_p(raw.data_ptr()),
                           C.c_void_p(binc.ctypes.data), _fp(fdeg), _fp(fexp), None)
    if rc:
        raise RuntimeError(f"RvPhantomFrames failed ({rc}): {last_error()[1]}")
    d = abi.RvStackDesc()
    d.ixdim, d.nframes, d.nslices = W, views + 2, S
    d.bInc = C.cast(C.c_void_p(binc.ctypes.data), C.POINTER(C.c_char))
    d.fdeg, d.fexp = _fp(fdeg), _fp(fexp)
    sino = torch.empty_like(raw)
    rc = L.RvNormaliseStack(C.byref(d), C.c_void_p(raw.data_ptr()), C.c_void_p(sino.data_ptr()), None)
    if rc:
        raise RuntimeError(f"RvNormaliseStack failed ({rc}): {last_error()[1]}")
    return Scan(raw, sino, binc, fdeg, centre)


def getaxis_grid_centre(scan: Scan, row: int = 1) -> float:
    """GetAxis on the 0-degree frame, the last sample frame (180 degrees minus a step) and the
    first flat; returns the ri->center of detector row `row` (user centre + 0.5)."""
    h = scan.raw.cpu().numpy().view(np.uint16)
    views = len(scan.bInc) - 2
    f0, f1, fl = (np.ascontiguousarray(h[k]) for k in (1, views, 0))
    u16 = lambda a: a.ctypes.data_as(C.POINTER(C.c_ushort))  # noqa: E731
    a, g, o = C.c_double(), C.c_double(), C.c_double()
    S, W = h.shape[1], h.shape[2]
    rc = lib().RvGetAxis(u16(f0), u16(f1), u16(fl), W, S, 0, C.byref(a), C.byref(g), C.byref(o))
    if rc:
        raise RuntimeError(f"RvGetAxis failed ({rc}): {last_error()[1]}")
    return a.value + g.value * row + 0.5


def sweep_filter(W: int) -> np.ndarray:
    return set_filter(abi.FILT_HAN, dims(W).ndim, cutoff=0.25)


def search(net, scan: Scan, grid_centre: float, F: np.ndarray, half_range: int = 40, step: float = 0.5,
           window: int = 2, sigma_max: float = 6.0) -> abi.RvCentreSearchResult:
    """RvCentreSearch on rows 0..3 (network) and row 1 (sweep); net None = the plain full sweep."""
    S, W = scan.sino.shape[1], scan.sino.shape[2]
    r = abi.RvCentreSearchResult()
    rc = lib().RvCentreSearch(net, C.c_void_p(scan.sino.data_ptr()), S, W, len(scan.bInc),
                              C.c_void_p(scan.bInc.ctypes.data), _fp(scan.fdeg), 0, 1, _fp(F), grid_centre, half_range,
                              step, window, sigma_max, C.byref(r), None)
    if rc:
        raise RuntimeError(f"RvCentreSearch failed ({rc}): {last_error()[1]}")
    return r


class CentreNet:
    """RvCentreNet at the production input size (4 x 256 x 512)."""

    def __init__(self, batch: int = 32, seed: int = 7):
        self.h = C.c_void_p()
        rc = lib().RvCentreNetCreate(256, 512, batch, seed, C.byref(self.h))
        if rc:
            raise RuntimeError(f"RvCentreNetCreate failed ({rc}): {last_error()[1]}")
        self.batch = batch

    @property
    def nparams(self) -> int:
        return lib().RvCentreNetNumParams(self.h)

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.nparams, np.float32)
        lib().RvCentreNetGetParams(self.h, _fp(p))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.nparams
        lib().RvCentreNetSetParams(self.h, _fp(p))

    def close(self):
        if self.h:
            lib().RvCentreNetDestroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_samples(desc: abi.RvCentreTrainDesc, first: int, count: int):
    """(X [count,4,256,512] bf16, Y [count] float) on the device."""
    import torch
    X = torch.empty((count, 4, 256, 512), dtype=torch.bfloat16, device="cuda")
    Y = torch.empty(count, dtype=torch.float32, device="cuda")
    rc = lib().RvCentreNetMakeSamples(C.byref(desc), first, count, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()),
                                      None)
    if rc:
        raise RuntimeError(f"RvCentreNetMakeSamples failed ({rc}): {last_error()[1]}")
    return X, Y


def fit(net: CentreNet, X, Y, ntrain: int, nval: int, epochs: int, lr_max: float = 1e-3, lr_min: float = 1e-5,
        seed: int = 3) -> np.ndarray:
    stats = np.zeros(4, np.float32)
    rc = lib().RvCentreNetFit(net.h, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()), ntrain, nval, epochs,
                              net.batch, lr_max, lr_min, seed, _fp(stats), None)
    if rc:
        raise RuntimeError(f"RvCentreNetFit failed ({rc}): {last_error()[1]}")
    return stats


def scan_input(scan: Scan):
    """The network input of a full scan (its 256 chosen views, rows 0..3) as a device tensor."""
    import torch
    frames = np.flatnonzero(scan.bInc & 1)
    V = len(frames)
    f256 = np.array([frames[min(V - 1, int(math.floor(r * V / 256.0 + 0.5)))] for r in range(256)], np.int32)
    x = torch.empty((1, 4, 256, 512), dtype=torch.bfloat16, device="cuda")
    S, W = scan.sino.shape[1], scan.sino.shape[2]
    rc = lib().RvCentreNetInput(C.c_void_p(scan.sino.data_ptr()), S, W, f256.ctypes.data_as(C.POINTER(C.c_int)), 0,
                                C.c_void_p(x.data_ptr()), None)
    if rc:
        raise RuntimeError(f"RvCentreNetInput failed ({rc}): {last_error()[1]}")
    return x
