"""Batched queue: uneven datasets (detector widths, view counts, centres, zoom) through one
persistent back-projection per wave and a captured CUDA graph; every slice must equal the
oracle's (the reference CPU routine restated) bit for bit."""
import ctypes as C

import numpy as np
import pytest

import recview_gb300 as rv
from recview_gb300 import abi, phantom
from recview_gb300.reconst import ReconInfo

pytestmark = pytest.mark.gpu

# (seed, W, V, slices, centre, iInterpolation)
DATASETS = [(1, 128, 120, 3, 61.7, 2), (2, 96, 90, 2, 50.3, 3), (3, 200, 150, 2, 97.2, 2), (4, 64, 60, 4, 30.9, 4)]


def _desc(W, nframes, S, cen, interp, bInc, fdeg, fexp, F):
    d = abi.RvStackDesc()
    d.ixdim, d.iInterpolation, d.center, d.nframes, d.nslices = W, interp, cen, nframes, S
    d.bInc = C.cast(C.c_void_p(bInc.ctypes.data), C.POINTER(C.c_char))
    d.fdeg = fdeg.ctypes.data_as(C.POINTER(C.c_float))
    d.fexp = fexp.ctypes.data_as(C.POINTER(C.c_float))
    d.fFilter = F.ctypes.data_as(C.POINTER(C.c_float))
    d.mode = abi.MODE_REF
    return d


def _oracle_stack(oracle, raw, bInc, fdeg, fexp, cen, F, interp):
    r = raw.copy()
    S = raw.shape[1]
    ri = ReconInfo(r.view(np.int16), fdeg, bInc, center=0, fexp=fexp, iMultiplex=S, maxSinogrLen=raw.shape[0])
    oracle.generate_sinogram(ri)
    return np.stack([oracle.reconstruct(ReconInfo(r.view(np.int16), fdeg, bInc, center=cen, fFilter=F,
                                                  iInterpolation=interp, iMultiplex=S, iOffset=s,
                                                  maxSinogrLen=r.shape[0] * S, nviews=raw.shape[0] - 1), threads=8)
                     for s in range(S)])


@pytest.fixture(scope="module")
def datasets(oracle):
    out = []
    for seed, W, V, S, cen, interp in DATASETS:
        raw, bInc, fdeg, fexp, _ = phantom.raw_stack(seed, W, V, S, cen, n_ellipsoids=8)
        F = oracle.set_filter(abi.FILT_SHEPP, rv.dims(W, interp).ndim)
        want = _oracle_stack(oracle, raw, bInc, fdeg, fexp, cen, F, interp)
        out.append((raw, bInc, fdeg, fexp, F, cen, interp, W, S, want))
    return out


@pytest.mark.parametrize("budget_mb,autotune,pinned,grid", [(None, False, None, False), (16, False, None, False),
                                                            (None, True, None, False),
                                                            (None, False, [18, 16, 0, 11], False),
                                                            (16, False, [16, 18, 9, 18], False),
                                                            (16, False, [18, 16, 0, 18], True)])
def test_queue_matches_oracle(gpu, datasets, monkeypatch, budget_mb, autotune, pinned, grid):
    torch = pytest.importorskip("torch")
    if budget_mb:
        monkeypatch.setenv("RV_TABLE_BUDGET_MB", str(budget_mb))   # several waves
    if grid:   # every group takes the regular grid launches per part instead of the persistent kernel
        monkeypatch.setenv("RV_QUEUE_GRID_TILES", "1")
    L = rv.lib()
    q = C.c_void_p()
    assert L.RvQueueCreate(C.byref(q)) == 0
    keep, outs = [], []
    try:
        for raw, bInc, fdeg, fexp, F, cen, interp, W, S, want in datasets:
            d_raw = torch.from_numpy(raw.view(np.int16)).cuda()
            npix = rv.dims(W, interp).ixdimp
            d_out = torch.full((S, npix, npix), -1, dtype=torch.int32, device="cuda")
            desc = _desc(W, raw.shape[0] - 1, S, cen, interp, bInc, fdeg, fexp, F)
            assert L.RvQueueAdd(q, C.byref(desc), C.c_void_p(d_raw.data_ptr()), C.c_void_p(d_out.data_ptr())) == 0, \
                rv.last_error()
            keep.append(d_raw)
            outs.append((d_out, want))
        if autotune:
            chosen = C.c_int(-1)
            assert L.RvQueueAutotune(q, None, C.byref(chosen)) == 0, rv.last_error()
            assert 0 <= chosen.value <= 21
            assert L.RvQueueItemVariant(q, 0) == chosen.value
            for i in range(len(datasets)):
                assert 0 <= L.RvQueueItemVariant(q, i) <= 21
        if pinned:   # datasets on different variants: one persistent launch per variant and wave
            for i, v in enumerate(pinned):
                assert L.RvQueueSetItemVariant(q, i, v) == 0
                assert L.RvQueueItemVariant(q, i) == v
            assert L.RvQueueSetItemVariant(q, 0, 22) == abi.RV_ERR_BAD_ARGUMENT
            assert L.RvQueueItemVariant(q, len(datasets)) == -1
        for run in range(2):   # first run captures the graph, second replays it
            for d_out, _ in outs:
                d_out.fill_(-1)
            assert L.RvQueueRun(q, None) == 0, rv.last_error()
            torch.cuda.synchronize()
            for d_out, want in outs:
                assert np.array_equal(d_out.cpu().numpy(), want), f"run {run}"
        assert L.RvQueueLastMs(q) > 0
        assert L.RvQueueUpdates(q) == sum(float(w.size) * (raw.shape[0] - 3) for (raw, *_r, w) in datasets)
    finally:
        L.RvQueueDestroy(q)


def test_queue_strip_assembly_dataset(gpu, oracle):
    """A dataset given as full-resolution frames with a trimmed region of interest and x2 zoom
    (the library trims; iTrim / iRawWidth) runs through the queue bit-exactly."""
    torch = pytest.importorskip("torch")
    F, T, interp, S, V = 240, 60, 3, 2, 90
    ixlen = oracle.L.rvo_bin_width(F, T, interp)
    raw, bInc, fdeg, fexp, _ = phantom.raw_stack(81, F, V, S, 121.4, n_ellipsoids=10)
    roi = oracle.bin_frames(raw, F, T, interp, S)
    cen = ixlen / 2.0 + 1.3
    Fl = oracle.set_filter(abi.FILT_SHEPP, rv.dims(ixlen, interp).ndim)
    want = _oracle_stack(oracle, roi, bInc, fdeg, fexp, cen, Fl, interp)
    L = rv.lib()
    q = C.c_void_p()
    assert L.RvQueueCreate(C.byref(q)) == 0
    try:
        d_raw = torch.from_numpy(raw.view(np.int16)).cuda()
        n = rv.dims(ixlen, interp).ixdimp
        d_out = torch.full((S, n, n), -1, dtype=torch.int32, device="cuda")
        desc = _desc(ixlen, raw.shape[0] - 1, S, cen, interp, bInc, fdeg, fexp, Fl)
        desc.iTrim, desc.iRawWidth = T, F
        assert L.RvQueueAdd(q, C.byref(desc), C.c_void_p(d_raw.data_ptr()), C.c_void_p(d_out.data_ptr())) == 0, \
            rv.last_error()
        assert L.RvQueueRun(q, None) == 0, rv.last_error()
        torch.cuda.synchronize()
        assert np.array_equal(d_out.cpu().numpy(), want)
    finally:
        L.RvQueueDestroy(q)
